// Host-side interface of the GB300 contact engine, used by the cntc_* API layer.
// Device memory for a set of patches is carved from one arena; the engine launches
// the influence-coefficient, spectrum and solve kernels on a caller-given stream.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <vector>
#include "engine.h"

namespace cgb {

// byte sizes of the per-patch device buffers: the io block (inputs and results) and the
// work area (influence coefficients, spectra, solver columns, FFT column buffers)
struct PatchSizes {
    size_t io, cf, spec64, spec32, wk, wki, rbuf, gscr, work;
};

// nblk: CTAs of the patch group (1: the patch is solved by one CTA); ncf: coefficient blocks
// (PatchDesc::ncf)
PatchSizes patch_sizes(int mx, int my, int fx, int fy, int nblk = 1, int ncf = 4);

// Assign the device pointers of d: io block at 'io' (patch_sizes().io bytes) and the work
// buffers inside [work, work + patch_sizes().work).
void carve_patch(PatchDesc &d, char *io, char *work);

// dynamic shared memory needed by the solve kernel for FFT half sizes fx, fy, for a patch
// solved by one CTA or (group) by a cooperative group of CTAs
size_t solve_smem_bytes(int fx, int fy, bool group = false);

// dynamic shared memory available to one CTA of the patch kernels on the current device
size_t max_dynamic_smem();

// CTAs of the group that solves an mx x my patch: 1 (one CTA) when the single-CTA plan fits
// and requested <= 1; otherwise a cooperative group of min(requested or one element per
// thread, co-resident CTAs of the device) CTAs.  requested: 0 automatic, 1 single CTA only,
// n >= 2 a group of (at most) n CTAs.  Returns -1 when neither form fits the device.
int group_size(int mx, int my, int fx, int fy, int requested);

// Launch the engine for n patches whose descriptors live in device memory (ddesc) and
// host memory (hdesc, same order).  compute_ic[i] != 0 requests influence coefficients and
// spectra for patch i.  The single-CTA patches are solved by one persistent launch, largest first.
// d_list is caller-owned device scratch for 3*n + 1 ints (the launch lists and the queue counter
// of the persistent solve) and must stay untouched until the launched work has finished.  Returns a cudaError_t value.
// Optional per-launch timing: when given, engine_run records ev[2k] before and ev[2k+1]
// after its k-th kernel launch on 'stream' and sets kind[k] (0 influence coefficients,
// 1 spectra, 2 patch solve).  The events are created by the caller.
struct EngineTimer {
    static constexpr int kMax = 32;
    cudaEvent_t ev[2 * kMax];
    int kind[kMax];
    int nlaunch = 0;
};

// All launches of a pass go to 'stream', so passes on different streams run concurrently.
int engine_run(const PatchDesc *hdesc, PatchDesc *ddesc, int n, const unsigned char *compute_ic,
               int *d_list, cudaStream_t stream, EngineTimer *timer = nullptr);

// engine_run in two parts, for passes that repeat on the same descriptors (the resident batch):
// engine_plan orders the patches and sizes the launches on the host (plan.all is the content of
// d_list, to be copied there by the caller); engine_launch only enqueues the pass's kernels on
// 'stream', with no host synchronisation, so that it can be captured into a CUDA graph.
struct EnginePlan {
    std::vector<int> all;               // d_list: influence list, spectra list, solve order
    int n_ic = 0, n_ics = 0, nsingle = 0, grid_solve = 0, kernels = 0;
    size_t maxsm = 0, sm_spec = 0, sm_solve = 0;
    dim3 ginf;
    struct Group { int k, nblk; size_t sm; void *gscr; bool ic; };
    std::vector<Group> groups;          // patch groups (cooperative launches)
};
int engine_plan(const PatchDesc *hdesc, int n, const unsigned char *compute_ic, EnginePlan &plan);
int engine_launch(const EnginePlan &plan, PatchDesc *ddesc, int *d_list, cudaStream_t stream,
                  EngineTimer *timer = nullptr);
// adds k to the count of kernel launches (launches replayed from a captured graph)
void count_launches(long long k);

// smallest 2^a 3^b 5^c 7^d >= n, following opt_fft_size (src/m_aijpj.f90:1022-1119)
int opt_fft_size(int n);

// count of this library's kernels launched since load (for benchmark accounting)
long long kernel_launch_count();

// subsurface elastic field of the surface tractions (subsurf.cu, m_subsurf.f90).  Host arrays;
// per point kSubsCols values: ux, uy, uz, sighyd, sigvm, sigtr, sigma1..3, sig[3][3] row by row.
// Points with z >= 0 lie in body 1, z < 0 in body 2.
struct SubsLoad {
    int mx, my;
    double dx, dy, xc1, yc1;          // grid: spacing and centre of the first element
    const double *pn, *px, *py;       // tractions of body 1, mx*my each (x fastest)
    double gg[2], poiss[2];           // the two bodies
};
constexpr int kSubsCols = 18;
// at npts arbitrary points xyz[3 q ..]
int subs_points(const SubsLoad &L, int npts, const double *xyz, double *out);
// at the element centres (ixs[a], iys[b]) (1-based, x fastest) at depth zw
int subs_depth(const SubsLoad &L, double zw, int nx, const int *ixs, int ny, const int *iys, double *out);

} // namespace cgb
