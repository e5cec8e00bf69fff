// Host-side interface of the GB300 contact engine, used by the cntc_* API layer.
// Device memory for a set of patches is carved from one arena; the engine launches
// the influence-coefficient, spectrum and solve kernels on a caller-given stream.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include "engine.h"

namespace cgb {

// byte sizes of the per-patch device buffers: the io block (inputs and results) and the
// work area (influence coefficients, spectra, solver columns, FFT column buffers)
struct PatchSizes {
    size_t io, cf, spec64, spec32, wk, wki, rbuf, work;
};

PatchSizes patch_sizes(int mx, int my, int fx, int fy);

// Assign the device pointers of d: io block at 'io' (patch_sizes().io bytes) and the work
// buffers inside [work, work + patch_sizes().work).
void carve_patch(PatchDesc &d, char *io, char *work);

// dynamic shared memory needed by the solve kernel for FFT half sizes fx, fy
size_t solve_smem_bytes(int fx, int fy);

// Launch the engine for n patches whose descriptors live in device memory (ddesc) and
// host memory (hdesc, same order).  compute_ic[i] != 0 requests influence coefficients and
// spectra for patch i.  Patches are grouped by shared-memory class internally.
// d_list is caller-owned device scratch for 2*n ints and must stay untouched until the
// launched work has finished.  Returns a cudaError_t value.
// Optional per-launch timing: when given, engine_run records ev[2k] before and ev[2k+1]
// after its k-th kernel launch on 'stream' and sets kind[k] (0 influence coefficients,
// 1 spectra, 2 patch solve).  The events are created by the caller.
struct EngineTimer {
    static constexpr int kMax = 32;
    cudaEvent_t ev[2 * kMax];
    int kind[kMax];
    int nlaunch = 0;
};

int engine_run(const PatchDesc *hdesc, PatchDesc *ddesc, int n, const unsigned char *compute_ic,
               int *d_list, cudaStream_t stream, EngineTimer *timer = nullptr);

// smallest 2^a 3^b 5^c 7^d >= n, following opt_fft_size (src/m_aijpj.f90:1022-1119)
int opt_fft_size(int n);

// count of this library's kernels launched since load (for benchmark accounting)
long long kernel_launch_count();

} // namespace cgb
