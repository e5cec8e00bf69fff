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
// Lines are transformed by line workers: the warps of the CTA for patches solved by one CTA,
// or the CTAs of the group (one CTA per line) for large patches.
//
//   step A  rows:    pairs of real rows (iy, iy+1) packed as one complex row, FFT over NX,
//                    split into two Hermitian half spectra, stored column-major R[kx][iy]
//   step B  columns: per kx, FFT over NY (only my non-zero inputs), multiply by the kernel
//                    spectrum (2x2 block for tangential products), inverse FFT, keep the my
//                    output rows, write back in place
//   step C  rows:    inverse of step A, real outputs ix < mx scaled by ga_inv / (NX NY)
//
// The full NX x NY spectrum is never stored: step B keeps one column in shared memory.
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
    C<T> *wbuf;             // shared: per line worker 4 * max(NX,NY)
    int wstride;            // complex elements per worker buffer region
    Lines L;                // line workers
    C<T> *R0, *R1;          // global: nkx * my each, column-major [kx][iy]
    double scale;           // ga_inv / (NX NY)
    long long *tacc;        // shared accumulator of cycles spent in convolutions (may be null)
    long long *tacc2;       // second cycle accumulator (may be null)
    double *bacc;           // shared accumulator of algorithmic bytes (may be null)
};

// step A: forward row transforms of ncomp real inputs (element-major, mx*my doubles each)
// into R0 (and R1).  'sel' optionally zeroes inputs outside a mask (mask[i] >= sel_lo).
template <typename T, typename IO>
__device__ __noinline__ void conv_rows_fwd(const Conv<T> &cv, const IO *in0, const IO *in1, int ncomp) {
    const Lines &L = cv.L;
    const int lane = L.lane, nl = L.nl;
    const int NX = cv.NX, mx = cv.mx, my = cv.my, nkx = cv.nkx;
    C<T> *a = cv.wbuf + L.widx * cv.wstride;
    C<T> *b = a + NX;
    const int npair = (my + 1) / 2;
    for (int comp = 0; comp < ncomp; comp++) {
        const IO *in = comp == 0 ? in0 : in1;
        C<T> *R = comp == 0 ? cv.R0 : cv.R1;
        for (int pr = L.w0; pr < npair; pr += L.nw) {
            const int iy0 = 2 * pr, iy1 = 2 * pr + 1;
            const bool has1 = iy1 < my;
            for (int ix = lane; ix < NX; ix += nl) {
                T re = 0, im = 0;
                if (ix < mx) {
                    re = (T)in[iy0 * mx + ix];
                    if (has1) im = (T)in[iy1 * mx + ix];
                }
                a[ix] = mkc<T>(re, im);
            }
            C<T> *z = line_fft<T>(a, b, cv.px, cv.twx, -1, lane, nl, L.blk);
            for (int k = lane; k < nkx; k += nl) {
                C<T> zk = z[k], zn = z[(NX - k) % NX];
                // A = (Z[k] + conj Z[n-k]) / 2 ; B = (Z[k] - conj Z[n-k]) / (2i)
                C<T> A = mkc<T>((T)0.5 * (zk.x + zn.x), (T)0.5 * (zk.y - zn.y));
                C<T> B = mkc<T>((T)0.5 * (zk.y + zn.y), (T)0.5 * (zn.x - zk.x));
                R[(size_t)k * my + iy0] = A;
                if (has1) R[(size_t)k * my + iy1] = B;
            }
            line_sync(L.blk);
        }
    }
}

// step B: per column kx, forward FFT over NY, multiply by the kernel spectrum, inverse FFT.
// ncomp == 1: u = K0 p ; ncomp == 2: (ux,uy) = [[Kxx, Kxy],[Kxy, Kyy]] (px,py) with
// K = {Kxx, Kxy, Kyy}.  Kernel blocks are (fx+1) x (fy+1) real, [kx][ky].
template <typename T>
__device__ __noinline__ void conv_cols(const Conv<T> &cv, int ncomp, const T *K0, const T *K1, const T *K2) {
    const Lines &L = cv.L;
    const int lane = L.lane, nl = L.nl;
    const int NY = cv.NY, my = cv.my, nkx = cv.nkx, fy = cv.fy;
    C<T> *a0 = cv.wbuf + L.widx * cv.wstride;
    C<T> *b0 = a0 + NY;
    C<T> *a1 = b0 + NY;
    C<T> *b1 = a1 + NY;
    for (int kx = L.w0; kx < nkx; kx += L.nw) {
        C<T> *col0 = cv.R0 + (size_t)kx * my;
        C<T> *col1 = cv.R1 + (size_t)kx * my;
        for (int iy = lane; iy < NY; iy += nl) {
            a0[iy] = iy < my ? col0[iy] : mkc<T>(0, 0);
            if (ncomp == 2) a1[iy] = iy < my ? col1[iy] : mkc<T>(0, 0);
        }
        C<T> *z0 = line_fft<T>(a0, b0, cv.py, cv.twy, -1, lane, nl, L.blk);
        C<T> *z1 = (ncomp == 2) ? line_fft<T>(a1, b1, cv.py, cv.twy, -1, lane, nl, L.blk) : nullptr;
        const size_t kb = (size_t)kx * (fy + 1);
        for (int ky = lane; ky < NY; ky += nl) {
            const int kq = ky <= fy ? ky : NY - ky;
            if (ncomp == 1) {
                T k0 = K0[kb + kq];
                z0[ky] = cscale<T>(z0[ky], k0);
            } else {
                // the xy kernel is odd in y: its real spectrum is odd in ky
                T kxx = K0[kb + kq], kxy = (ky <= fy) ? K1[kb + kq] : -K1[kb + kq], kyy = K2[kb + kq];
                C<T> p0 = z0[ky], p1 = z1[ky];
                z0[ky] = cadd<T>(cscale<T>(p0, kxx), cscale<T>(p1, kxy));
                z1[ky] = cadd<T>(cscale<T>(p0, kxy), cscale<T>(p1, kyy));
            }
        }
        C<T> *o0 = (z0 == a0) ? b0 : a0;
        C<T> *r0 = line_fft<T>(z0, o0, cv.py, cv.twy, +1, lane, nl, L.blk);
        C<T> *r1 = nullptr;
        if (ncomp == 2) {
            C<T> *o1 = (z1 == a1) ? b1 : a1;
            r1 = line_fft<T>(z1, o1, cv.py, cv.twy, +1, lane, nl, L.blk);
        }
        for (int iy = lane; iy < my; iy += nl) {
            col0[iy] = r0[iy];
            if (ncomp == 2) col1[iy] = r1[iy];
        }
        line_sync(L.blk);
    }
}

// output modes of step C
constexpr int OUT_ALL = 0;      // u[i] = val for all elements
constexpr int OUT_INT = 1;      // u[i] = val where igs >= Adhes (AllInt), others untouched
constexpr int OUT_ADDINT = 2;   // u[i] += val where igs >= Adhes

// step C: inverse row transforms, writes u (element-major doubles)
template <typename T, typename IO>
__device__ __noinline__ void conv_rows_inv(const Conv<T> &cv, IO *out0, IO *out1, int ncomp, int mode,
                              const int *igs) {
    const Lines &L = cv.L;
    const int lane = L.lane, nl = L.nl;
    const int NX = cv.NX, mx = cv.mx, my = cv.my, nkx = cv.nkx;
    C<T> *a = cv.wbuf + L.widx * cv.wstride;
    C<T> *b = a + NX;
    const int npair = (my + 1) / 2;
    const T sc = (T)cv.scale;
    for (int comp = 0; comp < ncomp; comp++) {
        IO *out = comp == 0 ? out0 : out1;
        const C<T> *R = comp == 0 ? cv.R0 : cv.R1;
        for (int pr = L.w0; pr < npair; pr += L.nw) {
            const int iy0 = 2 * pr, iy1 = 2 * pr + 1;
            const bool has1 = iy1 < my;
            for (int k = lane; k < NX; k += nl) {
                C<T> A, B;
                if (k < nkx) {
                    A = R[(size_t)k * my + iy0];
                    B = has1 ? R[(size_t)k * my + iy1] : mkc<T>(0, 0);
                } else {
                    A = cconj<T>(R[(size_t)(NX - k) * my + iy0]);
                    B = has1 ? cconj<T>(R[(size_t)(NX - k) * my + iy1]) : mkc<T>(0, 0);
                }
                // Z = A + i B
                a[k] = mkc<T>(A.x - B.y, A.y + B.x);
            }
            C<T> *z = line_fft<T>(a, b, cv.px, cv.twx, +1, lane, nl, L.blk);
            for (int ix = lane; ix < mx; ix += nl) {
                const int i0 = iy0 * mx + ix;
                const IO v0 = (IO)(z[ix].x * sc);
                if (mode == OUT_ALL) out[i0] = v0;
                else if (igs[i0] >= Adhes) out[i0] = (mode == OUT_INT) ? v0 : out[i0] + v0;
                if (has1) {
                    const int i1 = iy1 * mx + ix;
                    const IO v1 = (IO)(z[ix].y * sc);
                    if (mode == OUT_ALL) out[i1] = v1;
                    else if (igs[i1] >= Adhes) out[i1] = (mode == OUT_INT) ? v1 : out[i1] + v1;
                }
            }
            line_sync(L.blk);
        }
    }
}

// full product u = A p.  Synchronises the patch group before and after.
template <typename T, typename IO = double>
__device__ void convolve(const Conv<T> &cv, const IO *in0, const IO *in1, IO *out0, IO *out1,
                         int ncomp, const T *K0, const T *K1, const T *K2, int mode, const int *igs) {
    gsync();
    long long t0 = clock64();
    conv_rows_fwd<T, IO>(cv, in0, in1, ncomp);
    gsync();
    conv_cols<T>(cv, ncomp, K0, K1, K2);
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
