// Device-side building blocks of the GB300 contact engine: complex arithmetic,
// element-division codes, the patch group context and the reductions.
//
// A patch is solved by a group of thread blocks (CTAs): one CTA for grids whose FFT lines
// fit the per-warp shared-memory buffers (the batched workloads), or a cooperative grid of
// CTAs for large grids.  Every scalar decision of the solver is made from a reduction over
// the whole group and is therefore uniform across it: within one CTA a deterministic
// block tree, across CTAs the per-CTA partials summed in rank order by every CTA.
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

// ---------------------------------------------------------------------------------------------
// patch group: the CTAs that solve one patch together.  nblk == 1 is the single-CTA solve;
// for nblk > 1 the CTAs are co-resident (cooperative launch) and meet at grid barriers.
// Group scratch in global memory: bar[0] arrivals, bar[1] generation, bar[2] error flag;
// part: two slots of nblk x kRedSlot partials (doubles), parti: the same for ints.
// ---------------------------------------------------------------------------------------------
constexpr int kRedSlot = 8;
constexpr long long kBarrierTimeoutNs = 20000000000LL;   // a barrier gives up after 20 s

struct GroupCtx {
    int nblk, rank, seq;
    unsigned *bar;
    double *part;
    int *parti;
};

__shared__ GroupCtx g_grp;

__host__ __device__ inline size_t group_scratch_bytes(int nblk) {
    return 256 + (size_t)2 * nblk * kRedSlot * (sizeof(double) + sizeof(int));
}

// set by every CTA at kernel start (thread 0), before its first barrier
__device__ inline void group_init(int nblk, int rank, void *scratch) {
    if (threadIdx.x == 0) {
        g_grp.nblk = nblk;
        g_grp.rank = rank;
        g_grp.seq = 0;
        g_grp.bar = (unsigned *)scratch;
        g_grp.part = (double *)((char *)scratch + 256);
        g_grp.parti = (int *)(g_grp.part + (size_t)2 * nblk * kRedSlot);
    }
    __syncthreads();
}

// element index of this thread within the group and the group's stride
__device__ __forceinline__ int gtid() { return g_grp.rank * kThreads + threadIdx.x; }
__device__ __forceinline__ int gstride() { return g_grp.nblk * kThreads; }
// one thread of the whole group (global writes that must happen once)
__device__ __forceinline__ bool glead() { return threadIdx.x == 0 && g_grp.rank == 0; }
__device__ __forceinline__ bool grouped() { return g_grp.nblk > 1; }

__device__ __forceinline__ long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return (long long)t;
}

// barrier of the group: a block barrier for one CTA; across CTAs a generation barrier on
// the group scratch with memory fences on both sides (writes before it are visible to all
// CTAs after it).  The wait is bounded: after kBarrierTimeoutNs the CTA sets the error flag
// and returns; once the flag is set no CTA waits any more, so the solve runs out within its
// iteration limits and the host reports the failure.
__device__ __noinline__ void gsync_grid() {
    if (threadIdx.x == 0) {
        volatile unsigned *vb = g_grp.bar;
        const unsigned gen = vb[1];
        __threadfence();
        const unsigned a = atomicAdd(g_grp.bar, 1u);
        if (a == (unsigned)g_grp.nblk - 1) {
            atomicExch(g_grp.bar, 0u);
            __threadfence();
            atomicAdd(g_grp.bar + 1, 1u);
        } else {
            const long long t0 = global_ns();
            while (vb[1] == gen && vb[2] == 0u) {
                __nanosleep(64);
                if (global_ns() - t0 > kBarrierTimeoutNs) { atomicExch(g_grp.bar + 2, 1u); break; }
            }
        }
        __threadfence();
    }
    __syncthreads();
    __threadfence();
}

__device__ __forceinline__ void gsync() {
    __syncthreads();
    if (g_grp.nblk > 1) gsync_grid();
}

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

// Combine the block results v[0..K) (held by every thread of each CTA) over the CTAs of the
// group: thread 0 of each CTA publishes its partials in the current slot, a grid barrier,
// then warp 0 of every CTA combines all CTAs' partials in rank order (fixed lane split and
// shuffle tree), so that every CTA obtains the same value.  op: 0 sum, 1 max, 2 min.
template <typename V, int K>
__device__ __forceinline__ void group_combine(RedSmem &s, V (&v)[K], V *bcast, int op) {
    if (g_grp.nblk <= 1) return;
    const int nb = g_grp.nblk, slot = g_grp.seq & 1;
    V *part = (sizeof(V) == 8) ? (V *)(void *)g_grp.part : (V *)(void *)g_grp.parti;
    part += (size_t)slot * nb * kRedSlot;
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < K; k++) part[g_grp.rank * kRedSlot + k] = v[k];
    }
    __syncthreads();
    gsync_grid();
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (w == 0) {
#pragma unroll
        for (int k = 0; k < K; k++) {
            V t = (op == 0) ? V(0) : __ldcg(part + k);
            for (int r = lane; r < nb; r += 32) {
                const V x = __ldcg(part + (size_t)r * kRedSlot + k);
                t = (op == 0) ? t + x : (op == 1 ? (t > x ? t : x) : (t < x ? t : x));
            }
            for (int o = 16; o > 0; o >>= 1) {
                const V y = __shfl_down_sync(0xffffffffu, t, o);
                t = (op == 0) ? t + y : (op == 1 ? (t > y ? t : y) : (t < y ? t : y));
            }
            if (lane == 0) bcast[k] = t;
        }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < K; k++) v[k] = bcast[k];
    if (threadIdx.x == 0) g_grp.seq++;
    __syncthreads();
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
    group_combine<double, K>(s, v, s.bcast_d, 0);
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
    group_combine<int, K>(s, v, s.bcast_i, 0);
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
    double r[1] = {s.bcast_d[0]};
    __syncthreads();
    group_combine<double, 1>(s, r, s.bcast_d, 1);
    return r[0];
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
    double r[1] = {s.bcast_d[0]};
    __syncthreads();
    group_combine<double, 1>(s, r, s.bcast_d, 2);
    return r[0];
}

} // namespace cgb
