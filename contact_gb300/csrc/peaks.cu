// FP64 and FP32 fused multiply-add peaks of the current device, measured with CUDA events.
//
// The patch-solve kernel is bound by arithmetic, not by memory: its working set stays in
// L1/L2 and GB300's FP64 rate is a small fraction of its FP32 rate.  Its roofline therefore
// needs the device's own FMA rates as denominators.  Each thread runs kChains independent
// FMA chains (enough to cover the pipeline latency) for a fixed number of rounds; the grid
// holds several CTAs per SM so that every SM sub-partition issues.
#include <cuda_runtime.h>
#include <stdint.h>

namespace cgb {

constexpr int kPeakThreads = 256;
constexpr int kChains = 8;

template <typename T>
__global__ void __launch_bounds__(kPeakThreads) k_fma_peak(T *sink, int rounds, T a, T b) {
    T v[kChains];
#pragma unroll
    for (int c = 0; c < kChains; c++) v[c] = (T)(threadIdx.x + c) * (T)1e-3;
    for (int r = 0; r < rounds; r++) {
#pragma unroll
        for (int c = 0; c < kChains; c++) v[c] = v[c] * a + b;
    }
    T s = 0;
#pragma unroll
    for (int c = 0; c < kChains; c++) s += v[c];
    // written only for an impossible value, so the chains are not removed as dead code
    if (s == (T)-1.2345e30) sink[blockIdx.x * kPeakThreads + threadIdx.x] = s;
}

// flop/s of kernel k_fma_peak<T> over the whole device: best of 3 timed launches after one
// warm-up launch.  Returns 0 on any CUDA error.
template <typename T>
static double fma_rate(int rounds) {
    int dev = 0, nsm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0.0;
    if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0.0;
    const int blocks = nsm * 8;
    T *sink = nullptr;
    if (cudaMalloc(&sink, sizeof(T) * (size_t)blocks * kPeakThreads) != cudaSuccess) return 0.0;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    double best = 0.0;
    for (int rep = 0; rep < 4; rep++) {
        cudaEventRecord(e0);
        k_fma_peak<T><<<blocks, kPeakThreads>>>(sink, rounds, (T)0.999999, (T)1e-7);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && ms > 0.f) {
            const double flops = 2.0 * kChains * (double)rounds * blocks * kPeakThreads;
            const double r = flops / (ms * 1e-3);
            if (r > best) best = r;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(sink);
    if (cudaGetLastError() != cudaSuccess) return 0.0;
    return best;
}

} // namespace cgb

// out[0]: FP64 FMA peak (TFLOP/s), out[1]: FP32 FMA peak (TFLOP/s) of the current device.
// Returns 0, or -1 when a measurement failed.
extern "C" int cntc_gb300_fmapeaks(double *out) {
    const double f64 = cgb::fma_rate<double>(2048);
    const double f32 = cgb::fma_rate<float>(16384);
    out[0] = f64 * 1e-12;
    out[1] = f32 * 1e-12;
    return (f64 > 0.0 && f32 > 0.0) ? 0 : -1;
}
