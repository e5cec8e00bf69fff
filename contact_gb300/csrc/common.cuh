// Device-side building blocks of the GB300 contact engine: complex arithmetic,
// element-division codes and block-level reductions.  One thread block (CTA)
// owns one contact patch; every scalar decision of the solver is made from a
// block reduction and is therefore uniform across the CTA.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace cgb {

// element-division codes of CONTACT (src/m_gridfunc.f90:29-37)
constexpr int Exter = 0, Adhes = 1, Slip = 2, Plast = 3;

constexpr int kThreads = 256;           // threads per patch CTA
constexpr int kWarps = kThreads / 32;

template <typename T> struct cplx_t;
template <> struct cplx_t<double> { typedef double2 type; };
template <> struct cplx_t<float> { typedef float2 type; };

template <typename T> using C = typename cplx_t<T>::type;

template <typename T> __device__ __forceinline__ C<T> mkc(T r, T i) { C<T> z; z.x = r; z.y = i; return z; }
template <typename T> __device__ __forceinline__ C<T> cadd(C<T> a, C<T> b) { return mkc<T>(a.x + b.x, a.y + b.y); }
template <typename T> __device__ __forceinline__ C<T> csub(C<T> a, C<T> b) { return mkc<T>(a.x - b.x, a.y - b.y); }
template <typename T> __device__ __forceinline__ C<T> cmul(C<T> a, C<T> b) {
    return mkc<T>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
template <typename T> __device__ __forceinline__ C<T> cconj(C<T> a) { return mkc<T>(a.x, -a.y); }
template <typename T> __device__ __forceinline__ C<T> cscale(C<T> a, T s) { return mkc<T>(a.x * s, a.y * s); }

// ---------------------------------------------------------------------------------------------
// block reductions (deterministic: fixed strided accumulation order + fixed tree)
// ---------------------------------------------------------------------------------------------
struct RedSmem {
    double d[kWarps * 4];
    int i[kWarps * 4];
    double bcast_d[4];
    int bcast_i[4];
};

__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ int warp_sumi(int v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double warp_max(double v) {
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ double warp_min(double v) {
    for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_down_sync(0xffffffffu, v, o));
    return v;
}

// sum of up to 4 doubles over the block, result broadcast to all threads
template <int K>
__device__ __forceinline__ void block_sum(RedSmem &s, double (&v)[K]) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < K; k++) v[k] = warp_sum(v[k]);
    if (lane == 0) {
#pragma unroll
        for (int k = 0; k < K; k++) s.d[k * kWarps + w] = v[k];
    }
    __syncthreads();
    if (w == 0) {
#pragma unroll
        for (int k = 0; k < K; k++) {
            double t = (lane < kWarps) ? s.d[k * kWarps + lane] : 0.0;
            for (int o = kWarps / 2; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
            if (lane == 0) s.bcast_d[k] = t;
        }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < K; k++) v[k] = s.bcast_d[k];
    __syncthreads();
}

__device__ __forceinline__ double block_sum1(RedSmem &s, double v) {
    double a[1] = {v};
    block_sum<1>(s, a);
    return a[0];
}

template <int K>
__device__ __forceinline__ void block_sumi(RedSmem &s, int (&v)[K]) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < K; k++) v[k] = warp_sumi(v[k]);
    if (lane == 0) {
#pragma unroll
        for (int k = 0; k < K; k++) s.i[k * kWarps + w] = v[k];
    }
    __syncthreads();
    if (w == 0) {
#pragma unroll
        for (int k = 0; k < K; k++) {
            int t = (lane < kWarps) ? s.i[k * kWarps + lane] : 0;
            for (int o = kWarps / 2; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
            if (lane == 0) s.bcast_i[k] = t;
        }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < K; k++) v[k] = s.bcast_i[k];
    __syncthreads();
}

__device__ __forceinline__ int block_sumi1(RedSmem &s, int v) {
    int a[1] = {v};
    block_sumi<1>(s, a);
    return a[0];
}

__device__ __forceinline__ double block_max1(RedSmem &s, double v) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    v = warp_max(v);
    if (lane == 0) s.d[w] = v;
    __syncthreads();
    if (w == 0) {
        double t = (lane < kWarps) ? s.d[lane] : -1e300;
        for (int o = kWarps / 2; o > 0; o >>= 1) t = fmax(t, __shfl_down_sync(0xffffffffu, t, o));
        if (lane == 0) s.bcast_d[0] = t;
    }
    __syncthreads();
    double r = s.bcast_d[0];
    __syncthreads();
    return r;
}

__device__ __forceinline__ double block_min1(RedSmem &s, double v) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    v = warp_min(v);
    if (lane == 0) s.d[w] = v;
    __syncthreads();
    if (w == 0) {
        double t = (lane < kWarps) ? s.d[lane] : 1e300;
        for (int o = kWarps / 2; o > 0; o >>= 1) t = fmin(t, __shfl_down_sync(0xffffffffu, t, o));
        if (lane == 0) s.bcast_d[0] = t;
    }
    __syncthreads();
    double r = s.bcast_d[0];
    __syncthreads();
    return r;
}

} // namespace cgb
