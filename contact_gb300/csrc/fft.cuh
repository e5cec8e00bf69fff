// Shared-memory mixed-radix FFT (radix 8/4/2/3/5/7, Stockham auto-sort) executed by one
// warp per 1-D transform, and the doubled-grid convolution u = A * p of CONTACT's
// fft_VecAijPj (src/m_aijpj.f90:712-1015) built from it.
//
// Convolution layout.  The patch has mx x my elements; the FFT grid is NX x NY with
// NX = 2*fx, NY = 2*fy and fx = opt_fft_size(mx) >= mx (likewise fy): the linear
// convolution over offsets |d| <= mx-1 then has no wrap-around.  Influence
// coefficients are placed at (dx mod NX, dy mod NY); their spectra are real and
// quadrant-symmetric (even/odd kernels), stored as (fx+1) x (fy+1) values per block.
//
// The convolution transforms its lines in batches: a CTA loads as many lines as its shared-
// memory buffer holds and runs each Stockham stage over all butterflies of the batch at once
// (batch_fft), so that every thread has work in every stage whatever the line length, and one
// block barrier per stage serves the whole batch.  Batches go round the CTAs of a patch group.
//
//   step A  rows:    pairs of real rows (iy, iy+1) packed as one complex row, FFT over NX,
//                    split into two Hermitian half spectra, stored column-major R[kx][iy]
//                    (written with the rows of a batch fastest, so that stores are coalesced)
//   step B  columns: per kx, FFT over NY (only my non-zero inputs), multiply by the kernel
//                    spectrum (2x2 block for tangential products), inverse FFT, keep the my
//                    output rows, write back in place
//   step C  rows:    inverse of step A, real outputs ix < mx scaled by ga_inv / (NX NY)
//
// The full NX x NY spectrum is never stored: step B keeps a batch of columns in shared memory.
// Single transforms by a warp or a CTA (line_fft) serve the set-up of the kernel spectra.
#pragma once
#include "common.cuh"

namespace cgb {

constexpr int kMaxStages = 16;

struct FftPlan {
    int n;
    int nst;
    int rad[kMaxStages];
};

__host__ __device__ inline void fft_factorize(int n, FftPlan &p) {
    p.n = n; p.nst = 0;
    int m = n;
    while (m % 8 == 0 && p.nst < kMaxStages) { p.rad[p.nst++] = 8; m /= 8; }
    while (m % 4 == 0 && p.nst < kMaxStages) { p.rad[p.nst++] = 4; m /= 4; }
    while (m % 2 == 0 && p.nst < kMaxStages) { p.rad[p.nst++] = 2; m /= 2; }
    while (m % 3 == 0 && p.nst < kMaxStages) { p.rad[p.nst++] = 3; m /= 3; }
    while (m % 5 == 0 && p.nst < kMaxStages) { p.rad[p.nst++] = 5; m /= 5; }
    while (m % 7 == 0 && p.nst < kMaxStages) { p.rad[p.nst++] = 7; m /= 7; }
    // remaining prime factors use the generic O(p^2) stage
    for (int f = 11; m > 1 && p.nst < kMaxStages; f += 2)
        while (m % f == 0 && p.nst < kMaxStages) { p.rad[p.nst++] = f; m /= f; }
    if (m != 1) p.nst = -1;   // unsupported size
}

// cos/sin(2 pi q / R) for the odd radices (mathematical constants)
__device__ __forceinline__ double root_cos(int R, int q) {
    if (R == 3) { const double c[3] = {1.0, -0.5, -0.5}; return c[q]; }
    if (R == 5) {
        const double c[5] = {1.0, 0.30901699437494742410, -0.80901699437494742410, -0.80901699437494742410,
                             0.30901699437494742410};
        return c[q];
    }
    const double c[7] = {1.0, 0.62348980185873353053, -0.22252093395631440429, -0.90096886790241912624,
                         -0.90096886790241912624, -0.22252093395631440429, 0.62348980185873353053};
    return c[q];
}
__device__ __forceinline__ double root_sin(int R, int q) {
    if (R == 3) { const double s[3] = {0.0, 0.86602540378443864676, -0.86602540378443864676}; return s[q]; }
    if (R == 5) {
        const double s[5] = {0.0, 0.95105651629515357212, 0.58778525229247312917, -0.58778525229247312917,
                             -0.95105651629515357212};
        return s[q];
    }
    const double s[7] = {0.0, 0.78183148246802980871, 0.97492791218182360702, 0.43388373911755812048,
                         -0.43388373911755812048, -0.97492791218182360702, -0.78183148246802980871};
    return s[q];
}

// small DFT of radix R on registers; dir = -1 forward, +1 inverse
template <typename T, int R>
__device__ __forceinline__ void dft_small(C<T> (&v)[8], int dir) {
    if (R == 2) {
        C<T> a = v[0], b = v[1];
        v[0] = cadd<T>(a, b); v[1] = csub<T>(a, b);
    } else if (R == 4) {
        C<T> a0 = cadd<T>(v[0], v[2]), a1 = csub<T>(v[0], v[2]);
        C<T> a2 = cadd<T>(v[1], v[3]), a3 = csub<T>(v[1], v[3]);
        C<T> a3r = (dir < 0) ? mkc<T>(a3.y, -a3.x) : mkc<T>(-a3.y, a3.x);   // * (dir i)
        v[0] = cadd<T>(a0, a2); v[2] = csub<T>(a0, a2);
        v[1] = cadd<T>(a1, a3r); v[3] = csub<T>(a1, a3r);
    } else if (R == 8) {
        const T h = (T)0.70710678118654752440;
        const T s = (T)dir;
        C<T> b[8];
#pragma unroll
        for (int r = 0; r < 4; r++) { b[r] = cadd<T>(v[r], v[r + 4]); b[r + 4] = csub<T>(v[r], v[r + 4]); }
        // b[4+r] *= w8^(r) with w8 = exp(dir i pi/4)
        b[5] = mkc<T>(h * (b[5].x - s * b[5].y), h * (b[5].y + s * b[5].x));
        b[6] = mkc<T>(-s * b[6].y, s * b[6].x);
        b[7] = mkc<T>(h * (-b[7].x - s * b[7].y), h * (-b[7].y + s * b[7].x));
        C<T> t0 = cadd<T>(b[0], b[2]), t1 = csub<T>(b[0], b[2]), t2 = cadd<T>(b[1], b[3]), t3 = csub<T>(b[1], b[3]);
        C<T> t3r = (dir < 0) ? mkc<T>(t3.y, -t3.x) : mkc<T>(-t3.y, t3.x);
        v[0] = cadd<T>(t0, t2); v[4] = csub<T>(t0, t2); v[2] = cadd<T>(t1, t3r); v[6] = csub<T>(t1, t3r);
        t0 = cadd<T>(b[4], b[6]); t1 = csub<T>(b[4], b[6]); t2 = cadd<T>(b[5], b[7]); t3 = csub<T>(b[5], b[7]);
        t3r = (dir < 0) ? mkc<T>(t3.y, -t3.x) : mkc<T>(-t3.y, t3.x);
        v[1] = cadd<T>(t0, t2); v[5] = csub<T>(t0, t2); v[3] = cadd<T>(t1, t3r); v[7] = csub<T>(t1, t3r);
    } else {
        // roots are compile-time constants of type T (R and q are known after unrolling);
        // the direction only flips the sign of the imaginary part
        const T sd = (dir < 0) ? T(-1) : T(1);
        C<T> out[8];
#pragma unroll
        for (int k = 0; k < R; k++) {
            C<T> acc = v[0];
#pragma unroll
            for (int r = 1; r < R; r++) {
                const int q = (r * k) % R;
                const T wc = (T)root_cos(R, q), ws = (T)root_sin(R, q);
                // root_sin holds sin(2 pi q / R); the root is exp(dir 2 pi i q / R)
                C<T> w = mkc<T>(wc, sd * ws);
                acc = cadd<T>(acc, cmul<T>(v[r], w));
            }
            out[k] = acc;
        }
#pragma unroll
        for (int k = 0; k < R; k++) v[k] = out[k];
    }
}

// one Stockham stage of radix R: src -> dst, Ns = product of previous radices
template <typename T, int R>
__device__ __forceinline__ void stockham_stage(const C<T> *src, C<T> *dst, int n, int Ns,
                                               const C<T> *tw, int dir, int lane, int nl) {
    const int nb = n / R;
    const int tstep = n / (Ns * R);
    for (int j = lane; j < nb; j += nl) {
        C<T> v[8];
        const int jm = j % Ns;
#pragma unroll
        for (int r = 0; r < R; r++) {
            C<T> a = src[j + r * nb];
            if (r > 0 && jm > 0) {
                C<T> w = tw[r * jm * tstep];          // r * jm * tstep < R * Ns * n / (Ns R) = n
                if (dir > 0) w = cconj<T>(w);
                a = cmul<T>(a, w);
            }
            v[r] = a;
        }
        dft_small<T, R>(v, dir);
        const int idx = (j / Ns) * Ns * R + jm;
#pragma unroll
        for (int r = 0; r < R; r++) dst[idx + r * Ns] = v[r];
    }
}

// generic radix-p Stockham stage for a prime p > 7: every (butterfly, output) pair is one
// O(p) sum; roots of unity come from the length-n table (W_p^e = tw[e * n/p])
template <typename T>
__device__ __forceinline__ void stockham_stage_generic(const C<T> *src, C<T> *dst, int n, int Ns, int R,
                                                       const C<T> *tw, int dir, int lane, int nl) {
    const int nb = n / R;
    const int tstep = n / (Ns * R);
    const int wstep = n / R;
    for (int t = lane; t < n; t += nl) {
        const int j = t % nb, k = t / nb;
        const int jm = j % Ns;
        C<T> acc = mkc<T>(0, 0);
        for (int r = 0; r < R; r++) {
            C<T> a = src[j + r * nb];
            if (r > 0 && jm > 0) {
                C<T> w = tw[(r * jm * tstep) % n];
                if (dir > 0) w = cconj<T>(w);
                a = cmul<T>(a, w);
            }
            C<T> wr = tw[(size_t)((r * k) % R) * wstep];
            if (dir > 0) wr = cconj<T>(wr);
            acc = cadd<T>(acc, cmul<T>(a, wr));
        }
        dst[(j / Ns) * Ns * R + jm + k * Ns] = acc;
    }
}

// ---------------------------------------------------------------------------------------------
// batched transforms: nl lines of length n at buf + l * ld, all butterflies of a stage spread
// over the threads of the CTA
// ---------------------------------------------------------------------------------------------
// Threads and (line, index) pairs of a batch: for rows no longer than the CTA, each thread
// keeps one index i of a row and visits every G-th line (G rows of the batch side by side);
// longer rows are strided over the CTA line by line.  Index arithmetic happens once per thread.
template <typename F>
__device__ __forceinline__ void for_lines(int nl, int len, F body) {
    const int bd = blockDim.x;
    if (len <= bd) {
        const int G = bd / len, l0 = threadIdx.x / len, i = threadIdx.x - l0 * len;
        if (l0 < G)
            for (int l = l0; l < nl; l += G) body(l, i);
    } else {
        for (int l = 0; l < nl; l++)
            for (int i = threadIdx.x; i < len; i += bd) body(l, i);
    }
}

// the same visit for a transfer from global to shared memory: four loads in flight per thread
// before their stores.  load(l, i) returns the value, store(l, i, v) places it.
template <typename V, typename FL, typename FS>
__device__ __forceinline__ void copy_lines(int nl, int len, FL load, FS store) {
    constexpr int U = 4;
    const int bd = blockDim.x;
    if (len <= bd) {
        const int G = bd / len, l0 = threadIdx.x / len, i = threadIdx.x - l0 * len;
        if (l0 >= G) return;
        for (int l = l0; l < nl; l += U * G) {
            V v[U];
#pragma unroll
            for (int u = 0; u < U; u++) if (l + u * G < nl) v[u] = load(l + u * G, i);
#pragma unroll
            for (int u = 0; u < U; u++) if (l + u * G < nl) store(l + u * G, i, v[u]);
        }
    } else {
        for (int l = 0; l < nl; l++)
            for (int i0 = threadIdx.x; i0 < len; i0 += U * bd) {
                V v[U];
#pragma unroll
                for (int u = 0; u < U; u++) if (i0 + u * bd < len) v[u] = load(l, i0 + u * bd);
#pragma unroll
                for (int u = 0; u < U; u++) if (i0 + u * bd < len) store(l, i0 + u * bd, v[u]);
            }
    }
}

// one radix-R Stockham stage over nl lines: each thread keeps its butterfly j of a line and
// the twiddles of j in registers
template <typename T, int R>
__device__ __forceinline__ void batch_stage(const C<T> *src, C<T> *dst, int ld, int n, int Ns, int nl,
                                            const C<T> *tw, int dir) {
    const int nb = n / R;
    const int tstep = n / (Ns * R);
    auto bfly = [&](int l, int j, const C<T> (&w)[8], int jm) {
        const C<T> *sl = src + (size_t)l * ld;
        C<T> *dl = dst + (size_t)l * ld;
        C<T> v[8];
#pragma unroll
        for (int r = 0; r < R; r++) {
            C<T> a = sl[j + r * nb];
            if (r > 0 && jm > 0) a = cmul<T>(a, w[r]);
            v[r] = a;
        }
        dft_small<T, R>(v, dir);
        const int idx = (j - jm) * R + jm;           // (j / Ns) Ns R + jm
#pragma unroll
        for (int r = 0; r < R; r++) dl[idx + r * Ns] = v[r];
    };
    auto twiddles = [&](int jm, C<T> (&w)[8]) {
#pragma unroll
        for (int r = 1; r < R; r++) {
            C<T> t = tw[r * jm * tstep];                 // r * jm * tstep < n
            w[r] = (dir > 0) ? cconj<T>(t) : t;
        }
    };
    const int bd = blockDim.x;
    if (nb <= bd) {
        const int G = bd / nb, l0 = threadIdx.x / nb, j = threadIdx.x - l0 * nb;
        if (l0 >= G) return;
        const int jm = j % Ns;
        C<T> w[8];
        twiddles(jm, w);
        for (int l = l0; l < nl; l += G) bfly(l, j, w, jm);
    } else {
        for (int j = threadIdx.x; j < nb; j += bd) {
            const int jm = j % Ns;
            C<T> w[8];
            twiddles(jm, w);
            for (int l = 0; l < nl; l++) bfly(l, j, w, jm);
        }
    }
}

template <typename T>
__device__ __forceinline__ void batch_stage_generic(const C<T> *src, C<T> *dst, int ld, int n, int Ns, int R, int nl,
                                                    const C<T> *tw, int dir) {
    const int nb = n / R;
    const int tstep = n / (Ns * R);
    const int wstep = n / R;
    const int total = nl * n;
    for (int t = threadIdx.x; t < total; t += blockDim.x) {
        const int l = t / n, tt = t - l * n;
        const int j = tt % nb, k = tt / nb;
        const int jm = j % Ns;
        const C<T> *sl = src + (size_t)l * ld;
        C<T> acc = mkc<T>(0, 0);
        for (int r = 0; r < R; r++) {
            C<T> a = sl[j + r * nb];
            if (r > 0 && jm > 0) {
                C<T> w = tw[(r * jm * tstep) % n];
                if (dir > 0) w = cconj<T>(w);
                a = cmul<T>(a, w);
            }
            C<T> wr = tw[(size_t)((r * k) % R) * wstep];
            if (dir > 0) wr = cconj<T>(wr);
            acc = cadd<T>(acc, cmul<T>(a, wr));
        }
        dst[(size_t)l * ld + (j - jm) * R + jm + k * Ns] = acc;
    }
}

// batched 1-D FFT by the whole CTA: nl lines (uniform over the CTA) of length p.n, line l at
// a + l * ld, scratch b of the same layout.  Returns the buffer holding the result, after a
// block barrier.  tw[k] = exp(-2 pi i k / n).
template <typename T>
__device__ __noinline__ C<T> *batch_fft(C<T> *a, C<T> *b, int ld, int nl, const FftPlan &p, const C<T> *tw,
                                        int dir) {
    int Ns = 1;
    C<T> *src = a, *dst = b;
    for (int s = 0; s < p.nst; s++) {
        const int R = p.rad[s];
        __syncthreads();
        switch (R) {
            case 8: batch_stage<T, 8>(src, dst, ld, p.n, Ns, nl, tw, dir); break;
            case 4: batch_stage<T, 4>(src, dst, ld, p.n, Ns, nl, tw, dir); break;
            case 2: batch_stage<T, 2>(src, dst, ld, p.n, Ns, nl, tw, dir); break;
            case 3: batch_stage<T, 3>(src, dst, ld, p.n, Ns, nl, tw, dir); break;
            case 5: batch_stage<T, 5>(src, dst, ld, p.n, Ns, nl, tw, dir); break;
            case 7: batch_stage<T, 7>(src, dst, ld, p.n, Ns, nl, tw, dir); break;
            default: batch_stage_generic<T>(src, dst, ld, p.n, Ns, R, nl, tw, dir); break;
        }
        Ns *= R;
        C<T> *t = src; src = dst; dst = t;
    }
    __syncthreads();
    return src;
}

// synchronisation of the threads that share one FFT line: a warp, or the whole CTA
__device__ __forceinline__ void line_sync(bool blk) {
    if (blk) __syncthreads(); else __syncwarp();
}

// 1-D FFT of length n by one line worker: a warp (lane = lane id, nl = 32) or the whole CTA
// (lane = thread id, nl = kThreads, blk).  Input in a, scratch b; returns the buffer holding
// the result, after a synchronisation of the worker.  tw[k] = exp(-2 pi i k / n).
template <typename T>
__device__ __noinline__ C<T> *line_fft(C<T> *a, C<T> *b, const FftPlan &p, const C<T> *tw, int dir, int lane, int nl,
                                       bool blk) {
    int Ns = 1;
    C<T> *src = a, *dst = b;
    for (int s = 0; s < p.nst; s++) {
        const int R = p.rad[s];
        line_sync(blk);
        switch (R) {
            case 8: stockham_stage<T, 8>(src, dst, p.n, Ns, tw, dir, lane, nl); break;
            case 4: stockham_stage<T, 4>(src, dst, p.n, Ns, tw, dir, lane, nl); break;
            case 2: stockham_stage<T, 2>(src, dst, p.n, Ns, tw, dir, lane, nl); break;
            case 3: stockham_stage<T, 3>(src, dst, p.n, Ns, tw, dir, lane, nl); break;
            case 5: stockham_stage<T, 5>(src, dst, p.n, Ns, tw, dir, lane, nl); break;
            case 7: stockham_stage<T, 7>(src, dst, p.n, Ns, tw, dir, lane, nl); break;
            default: stockham_stage_generic<T>(src, dst, p.n, Ns, R, tw, dir, lane, nl); break;
        }
        Ns *= R;
        C<T> *t = src; src = dst; dst = t;
    }
    line_sync(blk);
    return src;
}

// 1-D FFT of length n by one warp
template <typename T>
__device__ __forceinline__ C<T> *warp_fft(C<T> *a, C<T> *b, const FftPlan &p, const C<T> *tw, int dir) {
    return line_fft<T>(a, b, p, tw, dir, threadIdx.x & 31, 32, false);
}

// line workers of a patch: the warps of the CTA (single-CTA solve) or the CTAs of the group
// (cooperative solve of a large patch), each transforming one line at a time
struct Lines {
    int w0, nw;         // first line of this worker, number of workers (line stride)
    int lane, nl;       // thread index within the worker, threads per worker
    bool blk;           // worker = whole CTA
    int widx;           // index of the worker's buffer region in this CTA
};

__device__ inline Lines line_workers(bool blk) {
    Lines L;
    L.blk = blk;
    if (blk) { L.w0 = g_grp.rank; L.nw = g_grp.nblk; L.lane = threadIdx.x; L.nl = kThreads; L.widx = 0; }
    else { L.w0 = threadIdx.x >> 5; L.nw = kWarps; L.lane = threadIdx.x & 31; L.nl = 32; L.widx = threadIdx.x >> 5; }
    return L;
}

// twiddle table tw[k] = exp(-2 pi i k / n), filled by the whole block (a table in shared
// memory), or by the whole group (a table in global memory, blk)
template <typename T>
__device__ inline void make_twiddles(C<T> *tw, int n, bool blk = false) {
    const int k0 = blk ? gtid() : (int)threadIdx.x, ks = blk ? gstride() : (int)blockDim.x;
    for (int k = k0; k < n; k += ks) {
        double s, c;
        sincospi(-2.0 * (double)k / (double)n, &s, &c);
        tw[k] = mkc<T>((T)c, (T)s);
    }
}

// ---------------------------------------------------------------------------------------------
// Convolution context of one patch (everything in shared memory except R and the spectra)
// ---------------------------------------------------------------------------------------------
template <typename T>
struct Conv {
    int mx, my, NX, NY, fx, fy, nkx;
    FftPlan px, py;
    C<T> *twx, *twy;        // NX, NY: shared memory (single CTA) or global memory (group)
    C<T> *wbuf;             // shared: per line worker 4 * max(NX,NY) (kernel spectra set-up)
    int wstride;            // complex elements per worker buffer region
    Lines L;                // line workers (kernel spectra set-up)
    C<T> *cbuf;             // shared: the batch buffer of the convolution (both ping-pong halves)
    int ccap;               // complex elements of type T in cbuf
    C<T> *R0, *R1;          // global: nkx * my each, column-major [kx][iy]
    double scale;           // ga_inv / (NX NY)
    long long *tacc;        // shared accumulator of cycles spent in convolutions (may be null)
    long long *tacc2;       // second cycle accumulator (may be null)
    double *bacc;           // shared accumulator of algorithmic bytes (may be null)
};

// batches of the convolution go round the CTAs of the patch group (one CTA: all batches)
#define FOR_BATCH(bt, nbat) for (int bt = g_grp.rank; bt < (nbat); bt += g_grp.nblk)

// step A: forward row transforms of ncomp real inputs (element-major, mx*my each) into R0
// (and R1).  Lines are row pairs; a batch holds cap of them (stride NX + 1 complex).
template <typename T, typename IO>
__device__ __noinline__ void conv_rows_fwd(const Conv<T> &cv, const IO *in0, const IO *in1, int ncomp) {
    const int NX = cv.NX, mx = cv.mx, my = cv.my, nkx = cv.nkx;
    const int ld = NX + 1;
    const int cap = cv.ccap / (2 * ld);
    C<T> *a = cv.cbuf, *b = cv.cbuf + (size_t)cap * ld;
    const int npair = (my + 1) / 2;
    const int nbat = (npair + cap - 1) / cap;
    for (int comp = 0; comp < ncomp; comp++) {
        const IO *in = comp == 0 ? in0 : in1;
        C<T> *R = comp == 0 ? cv.R0 : cv.R1;
        FOR_BATCH(bt, nbat) {
            const int p0 = bt * cap, nl = min(cap, npair - p0);
            copy_lines<C<T>>(nl, NX,
                [&](int l, int ix) {
                    const int iy0 = 2 * (p0 + l);
                    T re = 0, im = 0;
                    if (ix < mx) {
                        re = (T)in[iy0 * mx + ix];
                        if (iy0 + 1 < my) im = (T)in[(iy0 + 1) * mx + ix];
                    }
                    return mkc<T>(re, im);
                },
                [&](int l, int ix, C<T> v) { a[(size_t)l * ld + ix] = v; });
            C<T> *z = batch_fft<T>(a, b, ld, nl, cv.px, cv.twx, -1);
            // A = (Z[k] + conj Z[n-k]) / 2 ; B = (Z[k] - conj Z[n-k]) / (2i); rows of the batch
            // fastest, so that consecutive threads store consecutive rows of a column
            for_lines(nkx, nl, [&](int k, int l) {
                const int iy0 = 2 * (p0 + l);
                const C<T> zk = z[(size_t)l * ld + k], zn = z[(size_t)l * ld + (k ? NX - k : 0)];
                R[(size_t)k * my + iy0] = mkc<T>((T)0.5 * (zk.x + zn.x), (T)0.5 * (zk.y - zn.y));
                if (iy0 + 1 < my) R[(size_t)k * my + iy0 + 1] = mkc<T>((T)0.5 * (zk.y + zn.y), (T)0.5 * (zn.x - zk.x));
            });
            __syncthreads();
        }
    }
}

// step B: per column kx, forward FFT over NY, multiply by the kernel spectrum, inverse FFT.
// ncomp == 1: u = K0 p ; ncomp == 2: (ux,uy) = [[Kxx, Kxy],[Kxy, Kyy]] (px,py) with
// K = {Kxx, Kxy, Kyy}.  Kernel blocks are (fx+1) x (fy+1) real, [kx][ky].  A batch holds cap
// columns, each as ncomp lines (stride NY + 1 complex).
// One component (ncomp = 1) may take a coupling kernel: kkind 1 (odd in x, even in y) and 2
// (even in x, odd in y) have imaginary spectra, K0 holds the imaginary part; kkind 3 (even in
// y) and 4 (odd in y) have no parity in x and complex spectra, K0 and K1 hold the real and
// imaginary parts.  ksign scales the product (the blocks zx = -xz, zy = -yz).
template <typename T>
__device__ __noinline__ void conv_cols(const Conv<T> &cv, int ncomp, const T *K0, const T *K1, const T *K2,
                                       int kkind = 0, T ksign = T(1)) {
    const int NY = cv.NY, my = cv.my, nkx = cv.nkx, fy = cv.fy;
    const int ld = NY + 1;
    const int cap = cv.ccap / (2 * ld * ncomp);
    C<T> *a = cv.cbuf, *b = cv.cbuf + (size_t)cap * ncomp * ld;
    const int nbat = (nkx + cap - 1) / cap;
    FOR_BATCH(bt, nbat) {
        const int k0 = bt * cap, nc = min(cap, nkx - k0), nl = nc * ncomp;
        copy_lines<C<T>>(nl, NY,
            [&](int line, int iy) {
                const int c = line / ncomp, comp = line - c * ncomp;
                return iy < my ? ((comp == 0 ? cv.R0 : cv.R1) + (size_t)(k0 + c) * my)[iy] : mkc<T>(0, 0);
            },
            [&](int line, int iy, C<T> v) { a[(size_t)line * ld + iy] = v; });
        C<T> *z = batch_fft<T>(a, b, ld, nl, cv.py, cv.twy, -1);
        for_lines(nc, NY, [&](int c, int ky) {
            const size_t kb = (size_t)(k0 + c) * (fy + 1);
            const int kq = ky <= fy ? ky : NY - ky;
            if (ncomp == 1 && kkind == 0) {
                z[(size_t)c * ld + ky] = cscale<T>(z[(size_t)c * ld + ky], K0[kb + kq]);
            } else if (ncomp == 1 && kkind <= 2) {
                // i s z, s odd in ky for kkind 2
                const T sv = ksign * ((kkind == 2 && ky > fy) ? -K0[kb + kq] : K0[kb + kq]);
                const C<T> v = z[(size_t)c * ld + ky];
                z[(size_t)c * ld + ky] = mkc<T>(-sv * v.y, sv * v.x);
            } else if (ncomp == 1) {
                // (kr + i ki) z, the spectrum mirrored in ky with the kernel's parity in y
                const T sg = (kkind == 4 && ky > fy) ? -ksign : ksign;
                const T kr = sg * K0[kb + kq], ki = sg * K1[kb + kq];
                const C<T> v = z[(size_t)c * ld + ky];
                z[(size_t)c * ld + ky] = mkc<T>(kr * v.x - ki * v.y, kr * v.y + ki * v.x);
            } else {
                // the xy kernel is odd in y: its real spectrum is odd in ky
                const T kxx = K0[kb + kq], kxy = (ky <= fy) ? K1[kb + kq] : -K1[kb + kq], kyy = K2[kb + kq];
                C<T> *z0 = z + (size_t)(2 * c) * ld, *z1 = z0 + ld;
                const C<T> p0 = z0[ky], p1 = z1[ky];
                z0[ky] = cadd<T>(cscale<T>(p0, kxx), cscale<T>(p1, kxy));
                z1[ky] = cadd<T>(cscale<T>(p0, kxy), cscale<T>(p1, kyy));
            }
        });
        C<T> *o = (z == a) ? b : a;
        C<T> *r = batch_fft<T>(z, o, ld, nl, cv.py, cv.twy, +1);
        for_lines(nl, my, [&](int line, int iy) {
            const int c = line / ncomp, comp = line - c * ncomp;
            ((comp == 0 ? cv.R0 : cv.R1) + (size_t)(k0 + c) * my)[iy] = r[(size_t)line * ld + iy];
        });
        __syncthreads();
    }
}

// output modes of step C
constexpr int OUT_ALL = 0;      // u[i] = val for all elements
constexpr int OUT_INT = 1;      // u[i] = val where igs >= Adhes (AllInt), others untouched
constexpr int OUT_ADDINT = 2;   // u[i] += val where igs >= Adhes
constexpr int OUT_ADDALL = 3;   // u[i] += val for all elements

// step C: inverse row transforms, writes u (element-major)
template <typename T, typename IO>
__device__ __noinline__ void conv_rows_inv(const Conv<T> &cv, IO *out0, IO *out1, int ncomp, int mode,
                              const int *igs) {
    const int NX = cv.NX, mx = cv.mx, my = cv.my, nkx = cv.nkx;
    const int ld = NX + 1;
    const int cap = cv.ccap / (2 * ld);
    C<T> *a = cv.cbuf, *b = cv.cbuf + (size_t)cap * ld;
    const int npair = (my + 1) / 2;
    const int nbat = (npair + cap - 1) / cap;
    const T sc = (T)cv.scale;
    for (int comp = 0; comp < ncomp; comp++) {
        IO *out = comp == 0 ? out0 : out1;
        const C<T> *R = comp == 0 ? cv.R0 : cv.R1;
        FOR_BATCH(bt, nbat) {
            const int p0 = bt * cap, nl = min(cap, npair - p0);
            // Z = A + i B from the half spectra of rows iy0, iy0 + 1 (rows of the batch fastest)
            copy_lines<C<T>>(NX, nl,
                [&](int k, int l) {
                    const int iy0 = 2 * (p0 + l);
                    const bool has1 = iy0 + 1 < my;
                    C<T> A, B;
                    if (k < nkx) {
                        A = R[(size_t)k * my + iy0];
                        B = has1 ? R[(size_t)k * my + iy0 + 1] : mkc<T>(0, 0);
                    } else {
                        A = cconj<T>(R[(size_t)(NX - k) * my + iy0]);
                        B = has1 ? cconj<T>(R[(size_t)(NX - k) * my + iy0 + 1]) : mkc<T>(0, 0);
                    }
                    return mkc<T>(A.x - B.y, A.y + B.x);
                },
                [&](int k, int l, C<T> v) { a[(size_t)l * ld + k] = v; });
            C<T> *z = batch_fft<T>(a, b, ld, nl, cv.px, cv.twx, +1);
            for_lines(nl, mx, [&](int l, int ix) {
                const int iy0 = 2 * (p0 + l);
                const C<T> zz = z[(size_t)l * ld + ix];
                const int i0 = iy0 * mx + ix;
                const bool has1 = iy0 + 1 < my;
                const IO v0 = (IO)(zz.x * sc), v1 = (IO)(zz.y * sc);
                if (mode == OUT_ALL) {
                    out[i0] = v0;
                    if (has1) out[i0 + mx] = v1;
                } else if (mode == OUT_ADDALL) {
                    out[i0] += v0;
                    if (has1) out[i0 + mx] += v1;
                } else {
                    const int g0 = igs[i0], g1 = has1 ? igs[i0 + mx] : Exter;
                    const IO o0 = (mode == OUT_ADDINT && g0 >= Adhes) ? out[i0] : IO(0);
                    const IO o1 = (mode == OUT_ADDINT && g1 >= Adhes) ? out[i0 + mx] : IO(0);
                    if (g0 >= Adhes) out[i0] = (mode == OUT_INT) ? v0 : o0 + v0;
                    if (g1 >= Adhes) out[i0 + mx] = (mode == OUT_INT) ? v1 : o1 + v1;
                }
            });
            __syncthreads();
        }
    }
}

// full product u = A p.  Synchronises the patch group before and after.
template <typename T, typename IO = double>
__device__ void convolve(const Conv<T> &cv, const IO *in0, const IO *in1, IO *out0, IO *out1,
                         int ncomp, const T *K0, const T *K1, const T *K2, int mode, const int *igs,
                         int kkind = 0, T ksign = T(1)) {
    gsync();
    long long t0 = clock64();
    conv_rows_fwd<T, IO>(cv, in0, in1, ncomp);
    gsync();
    conv_cols<T>(cv, ncomp, K0, K1, K2, kkind, ksign);
    gsync();
    conv_rows_inv<T, IO>(cv, out0, out1, ncomp, mode, igs);
    gsync();
    if (threadIdx.x == 0) {
        const long long dt = clock64() - t0;
        if (cv.tacc) *cv.tacc += dt;
        if (cv.tacc2) *cv.tacc2 += dt;
        // algorithmic bytes: inputs and outputs in their storage type, one real quadrant
        // spectrum per block in the working precision
        if (cv.bacc) {
            const int nblk = (K0 != nullptr) + (K1 != nullptr) + (K2 != nullptr);
            *cv.bacc += 2.0 * sizeof(IO) * ncomp * cv.mx * cv.my + (double)sizeof(T) * nblk * (cv.fx + 1) * (cv.fy + 1);
        }
    }
}

} // namespace cgb
