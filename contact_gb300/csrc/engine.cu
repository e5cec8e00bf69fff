// Kernels of the GB300 contact engine and their host-side launchers.
//
//   k_influence : Boussinesq-Cerruti influence coefficients, piecewise constant loading
//                 (elascf_pcwcns, src/m_visc.f90:431-604), blocks xx, xy, yy, zz
//   k_spectra   : real, quadrant-symmetric spectra of the coefficient blocks on the doubled
//                 FFT grid, and the FFT preconditioners ga^2 / spectrum (fft_makePrec,
//                 src/m_aijpj.f90:457-708, evaluated at the convolution's FFT size)
//   k_solve     : complete solve of one patch per thread block: right-hand sides and initial
//                 estimate (src/m_sdis.f90), Panagiotopoulos loop (src/m_scontc.f90:356-553)
//                 with NORM and TANG, output quantities (src/m_soutpt.f90:377-511)
#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>
#include "engine_api.h"
#include "solver.cuh"

namespace cgb {

static std::atomic<long long> g_launches(0);
long long kernel_launch_count() { return g_launches.load(); }

// ------------------------------------------------------------------------------------------
// influence coefficients
// ------------------------------------------------------------------------------------------
// corner (ix, iy) of the element grid, shifted by (xsh, ysh): the coordinates in the order of
// operations of elascf_pcwcns (m_visc.f90:470-489), so that the coefficients are bitwise
// those of a serial evaluation
__device__ inline void corner(int ix, int iy, double dx, double dy, double xsh, double ysh, double &x, double &y,
                              double &r) {
    x = ((double)(float)ix * dx + xsh) - 0.5 * dx;
    y = ((double)(float)iy * dy + ysh) - 0.5 * dy;
    r = sqrt(x * x + y * y);
}

// influence coefficients xx, xy (= yx), yy, zz of offset (ix, iy) for piecewise-constant
// loading (elascf_pcwcns, m_visc.f90:431-604) on grids shifted by (xsh, ysh); zero for rows
// below iy0 (single-row grids)
// c[0..3]: xx, xy, yy, zz; with cpl (K != 0, |ak| >= 1e-6 as in the reference) also c[4], c[5]:
// xz and yz (the terms with K of m_visc.f90:431-604, in its order of summation)
__device__ inline void influence_at(int ix, int iy, int iy0, double dx, double dy, double nu, double xsh, double ysh,
                                    double c[6], double ak = 0.0, bool cpl = false) {
    const double pi = 3.14159265358979323846;
    const double e1 = (1.0 - nu) / pi, e2 = 1.0 / pi, e3 = nu / pi;
    const double tolx = dx * 1e-10, tolx2 = dx * 1e-20;
    double c11 = 0, c12 = 0, c22 = 0, c33 = 0, c13 = 0, c23 = 0;
    if (iy >= iy0) {
        double x00, y00, r00, x01, y01, r01, x10, y10, r10, x11, y11, r11;
        corner(ix, iy, dx, dy, xsh, ysh, x00, y00, r00);
        corner(ix, iy + 1, dx, dy, xsh, ysh, x01, y01, r01);
        corner(ix + 1, iy, dx, dy, xsh, ysh, x10, y10, r10);
        corner(ix + 1, iy + 1, dx, dy, xsh, ysh, x11, y11, r11);
        c12 = 0.0 - e3 * r00;
        c12 = c12 + e3 * r01;
        c12 = c12 + e3 * r10;
        c12 = c12 - e3 * r11;
        double X0, X1, Y0, Y1;     // xly2y1(ix,iy), xly2y1(ix+1,iy), ylx2x1(ix,iy), ylx2x1(ix,iy+1)
        X0 = (fmin(fabs(y00 + r00), fabs(y01 + r01)) < tolx) ? 0.0 : x00 * log((y01 + r01) / (y00 + r00));
        X1 = (fmin(fabs(y10 + r10), fabs(y11 + r11)) < tolx) ? 0.0 : x10 * log((y11 + r11) / (y10 + r10));
        Y0 = (fmin(fabs(x00 + r00), fabs(x10 + r10)) < tolx) ? 0.0 : y00 * log((x10 + r10) / (x00 + r00));
        Y1 = (fmin(fabs(x01 + r01), fabs(x11 + r11)) < tolx) ? 0.0 : y01 * log((x11 + r11) / (x01 + r01));
        c33 = 0.0 - e1 * (X0 + Y0);
        c33 = c33 + e1 * (X1 + Y1);
        c11 = 0.0 - (e1 * X0 + e2 * Y0);
        c11 = c11 + (e1 * X1 + e2 * Y1);
        c22 = 0.0 - (e1 * Y0 + e2 * X0);
        c22 = c22 + (e1 * Y1 + e2 * X1);
        if (cpl) {
            // y log r + x atan(y / x) and x log r + y atan(x / y) at the four corners
            auto j5 = [&](double x, double y, double r) { return y * log(r) + x * atan(y / (x + tolx2)); };
            auto j6 = [&](double x, double y, double r) { return x * log(r) + y * atan(x / (y + tolx2)); };
            const double f = e2 * ak;
            c13 = 0.0 - f * j5(x00, y00, r00);
            c13 = c13 + f * j5(x01, y01, r01);
            c13 = c13 + f * j5(x10, y10, r10);
            c13 = c13 - f * j5(x11, y11, r11);
            c23 = 0.0 - f * j6(x00, y00, r00);
            c23 = c23 + f * j6(x01, y01, r01);
            c23 = c23 + f * j6(x10, y10, r10);
            c23 = c23 - f * j6(x11, y11, r11);
        }
    }
    c[0] = c11; c[1] = c12; c[2] = c22; c[3] = c33;
    if (cpl) { c[4] = c13; c[5] = c23; }
}

// grid: (blocks per patch, number of listed patches); list[] gives the patch indices
__global__ void __launch_bounds__(kThreads) k_influence(const PatchDesc *descs, const int *list) {
    const PatchDesc &d = descs[list[blockIdx.y]];
    const int mx = d.mx, my = d.my;
    const int total = 4 * mx * my;
    const int iy0 = (my == 1) ? 0 : -my;
    double *cf = const_cast<double *>(d.cf);
    const size_t bsz = (size_t)total;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
        const int ix = t % (2 * mx) - mx, iy = t / (2 * mx) - my;
        double c[6];
        const bool cpl = d.ncf >= 6;
        influence_at(ix, iy, iy0, d.dx, d.dy, d.nu, 0.0, 0.0, c, d.ak, cpl);
        cf[0 * bsz + t] = c[0];
        cf[1 * bsz + t] = c[1];
        cf[2 * bsz + t] = c[2];
        cf[3 * bsz + t] = c[3];
        if (cpl) {
            cf[4 * bsz + t] = c[4];
            cf[5 * bsz + t] = c[5];
        }
        if (d.ncf == 8) {
            // steady rolling: the coupling blocks of cs - cv, cv the grid shifted by one rolling
            // step (m_visc.f90:289-354), for u'(pn) of stang_rhs
            double v[6];
            influence_at(ix, iy, iy0, d.dx, d.dy, d.nu, cos(d.chi) * d.dq, sin(d.chi) * d.dq, v, d.ak, true);
            cf[6 * bsz + t] = c[4] - v[4];
            cf[7 * bsz + t] = c[5] - v[5];
        }
    }
}

// steady-rolling coefficients of ConvexGS: csv = cs - cv for blocks xx, xy, yy, where cv are
// the coefficients of the grid shifted by one rolling step (dq cos chi, dq sin chi)
// (m_visc.f90:289-354); written in the layout of cf to csv[3][2my][2mx]
__device__ __noinline__ void steady_coefs(const PatchDesc &d, double *csv) {
    const int mx = d.mx, my = d.my;
    const int total = 4 * mx * my;
    const int iy0 = (my == 1) ? 0 : -my;
    const double xsh = cos(d.chi) * d.dq, ysh = sin(d.chi) * d.dq;
    for (int t = gtid(); t < total; t += gstride()) {
        const int ix = t % (2 * mx) - mx, iy = t / (2 * mx) - my;
        double c[6];
        influence_at(ix, iy, iy0, d.dx, d.dy, d.nu, xsh, ysh, c);
        csv[0 * (size_t)total + t] = d.cf[0 * (size_t)total + t] - c[0];
        csv[1 * (size_t)total + t] = d.cf[1 * (size_t)total + t] - c[1];
        csv[2 * (size_t)total + t] = d.cf[2 * (size_t)total + t] - c[2];
    }
    gsync();
}

// coefficients of transient rolling cv: the grid shifted by one rolling step, formed as
// cs - (cs - shifted) like the reference's cv (m_visc.f90:289-354), blocks xx, xy, yy in the
// layout of cf
__device__ __noinline__ void transient_coefs(const PatchDesc &d, double *cv) {
    const int mx = d.mx, my = d.my;
    const int total = 4 * mx * my;
    const int iy0 = (my == 1) ? 0 : -my;
    const double xsh = cos(d.chi) * d.dq, ysh = sin(d.chi) * d.dq;
    for (int t = gtid(); t < total; t += gstride()) {
        const int ix = t % (2 * mx) - mx, iy = t / (2 * mx) - my;
        double c[6];
        influence_at(ix, iy, iy0, d.dx, d.dy, d.nu, xsh, ysh, c);
        for (int k = 0; k < 3; k++) {
            const double cs = d.cf[k * (size_t)total + t];
            cv[k * (size_t)total + t] = cs - (cs - c[k]);
        }
    }
    gsync();
}

// ------------------------------------------------------------------------------------------
// shared-memory plan of a patch block
// ------------------------------------------------------------------------------------------
struct SmemPlan {
    int NX, NY, nmax;
    size_t off_tw64x, off_tw64y, off_tw32x, off_tw32y, off_wbuf, total;
};

// Shared memory of a patch CTA: the convolution's batch buffer (cbuf) and, for a single CTA,
// the twiddle tables of the convolution size in FP64 and FP32 (a patch group keeps them in its
// scratch in global memory).  The batch buffer holds at least one ping-pong pair of the
// longest line for both components of a tangential product (64 (nmax + 1) bytes in FP64), and
// kConvBufBytes otherwise, so that two CTAs of the largest single-CTA grids share an SM.  The
// kernel-spectra set-up uses the same buffer for one CTA-wide line (4 nmax complex FP64).
constexpr size_t kConvBufBytes = 80 * 1024;

__host__ __device__ inline size_t conv_buf_bytes(int nmax) {
    const size_t need = (size_t)64 * (nmax + 1);
    return need > kConvBufBytes ? need : kConvBufBytes;
}

__host__ __device__ inline SmemPlan smem_plan(int fx, int fy, bool blk = false) {
    SmemPlan s;
    s.NX = 2 * fx; s.NY = 2 * fy; s.nmax = s.NX > s.NY ? s.NX : s.NY;
    size_t o = 0;
    if (blk) {
        s.off_tw64x = s.off_tw64y = s.off_tw32x = s.off_tw32y = 0;
        s.off_wbuf = 0;
        s.total = conv_buf_bytes(s.nmax);
        return s;
    }
    s.off_tw64x = o; o += (size_t)s.NX * 16;
    s.off_tw64y = o; o += (size_t)s.NY * 16;
    s.off_tw32x = o; o += (size_t)s.NX * 8;
    s.off_tw32y = o; o += (size_t)s.NY * 8;
    o = (o + 15) & ~(size_t)15;
    s.off_wbuf = o; o += conv_buf_bytes(s.nmax);
    s.total = o;
    return s;
}

// twiddle tables of a patch group inside its scratch (after the barrier and partials):
// convolution size NX, NY in FP64 and FP32, and the preconditioner period 2mx, 2my in FP64
struct GroupTw {
    size_t off64x, off64y, off32x, off32y, offpx, offpy, total;
};

__host__ __device__ inline GroupTw group_tw(int nblk, int mx, int my, int fx, int fy) {
    GroupTw g;
    size_t o = (group_scratch_bytes(nblk) + 255) & ~(size_t)255;
    g.off64x = o; o += (size_t)2 * fx * 16;
    g.off64y = o; o += (size_t)2 * fy * 16;
    g.off32x = o; o += (size_t)2 * fx * 8;
    g.off32y = o; o += (size_t)2 * fy * 8;
    g.offpx = o; o += (size_t)2 * mx * 16;
    g.offpy = o; o += (size_t)2 * my * 16;
    g.total = (o + 255) & ~(size_t)255;
    return g;
}

template <typename T>
__device__ inline Conv<T> make_conv(const PatchDesc &d, unsigned char *smraw, const SmemPlan &sp) {
    Conv<T> cv;
    const bool blk = d.nblk > 1;
    cv.mx = d.mx; cv.my = d.my; cv.fx = d.fx; cv.fy = d.fy;
    cv.NX = sp.NX; cv.NY = sp.NY; cv.nkx = d.fx + 1;
    fft_factorize(cv.NX, cv.px);
    fft_factorize(cv.NY, cv.py);
    cv.L = line_workers(blk);
    if (blk) {
        const GroupTw g = group_tw(d.nblk, d.mx, d.my, d.fx, d.fy);
        char *base = (char *)d.gscr;
        cv.twx = (C<T> *)(base + (sizeof(T) == 8 ? g.off64x : g.off32x));
        cv.twy = (C<T> *)(base + (sizeof(T) == 8 ? g.off64y : g.off32y));
    } else if (sizeof(T) == 8) {
        cv.twx = (C<T> *)(smraw + sp.off_tw64x);
        cv.twy = (C<T> *)(smraw + sp.off_tw64y);
    } else {
        cv.twx = (C<T> *)(smraw + sp.off_tw32x);
        cv.twy = (C<T> *)(smraw + sp.off_tw32y);
    }
    cv.wbuf = (C<T> *)(smraw + sp.off_wbuf);
    cv.wstride = 4 * sp.nmax;
    cv.cbuf = (C<T> *)(smraw + sp.off_wbuf);
    cv.ccap = (int)(conv_buf_bytes(sp.nmax) / sizeof(C<T>));
    C<T> *R = (C<T> *)d.rbuf;
    cv.R0 = R;
    cv.R1 = R + (size_t)cv.nkx * cv.my;
    cv.scale = 1.0 / (d.ga * (double)cv.NX * (double)cv.NY);
    cv.tacc = nullptr;
    cv.tacc2 = nullptr;
    cv.bacc = nullptr;
    return cv;
}

// doubles of complex scratch used by k_spectra before the spatial preconditioner kernel
__host__ __device__ inline size_t spectra_scratch_doubles(int mx, int my, int fx, int fy) {
    const size_t a = (size_t)(fx + 1) * 2 * fy * 2;      // conv-size spectrum rows
    const size_t b = (size_t)2 * mx * 2 * my * 2;        // 2mx x 2my complex period
    return a > b ? a : b;
}

template <typename T>
__device__ inline void make_ops(Ops<T> &op, const PatchDesc &d, unsigned char *smraw, const SmemPlan &sp) {
    op.cv = make_conv<T>(d, smraw, sp);
    const size_t ksz = (size_t)(d.fx + 1) * (d.fy + 1);
    const T *base = (sizeof(T) == 8) ? (const T *)(const void *)d.spec64 : (const T *)(const void *)d.spec32;
    for (int b = 0; b < kMaxSpectra; b++) op.K[b] = b < spectra_count(d.ncf) ? base + b * ksz : nullptr;
}

// ------------------------------------------------------------------------------------------
// spectra of the coefficient blocks and of the FFT preconditioners (one block per patch)
// ------------------------------------------------------------------------------------------
// real, quadrant-symmetric conv-size spectrum of a spatial block src (layout of cf:
// (dx + mx) + (dy + my) * 2mx); offsets |dx| <= mx-1, |dy| <= my-1 are placed at
// (dx mod NX, dy mod NY).  S: scratch of nkx * NY complex.
// imag: store the imaginary part instead of the real part (a block odd in exactly one of x, y,
// such as the coupling blocks xz, yz, has an imaginary spectrum; the coupling blocks of cs - cv,
// which have no parity in x, need both parts).
__device__ __noinline__ void block_spectrum(const Conv<double> &cv, const double *src, double2 *S, double *K64,
                                            float *K32, double2 *a, double2 *b, bool imag = false) {
    const int mx = cv.mx, my = cv.my, NX = cv.NX, NY = cv.NY, nkx = cv.nkx, fy = cv.fy;
    const Lines &L = cv.L;
    const int lane = L.lane, nl = L.nl;
    const int NONE = 1 << 30;
    gsync();
    for (int pr = L.w0; pr < NY / 2; pr += L.nw) {
        const int r0 = 2 * pr, r1 = 2 * pr + 1;
        const int dy0 = r0 < my ? r0 : (r0 > NY - my ? r0 - NY : NONE);
        const int dy1 = r1 < my ? r1 : (r1 > NY - my ? r1 - NY : NONE);
        for (int ix = lane; ix < NX; ix += nl) {
            const int dx = ix < mx ? ix : (ix > NX - mx ? ix - NX : NONE);
            double v0 = 0, v1 = 0;
            if (dx != NONE) {
                if (dy0 != NONE) v0 = src[(size_t)(dx + mx) + (size_t)(dy0 + my) * 2 * mx];
                if (dy1 != NONE) v1 = src[(size_t)(dx + mx) + (size_t)(dy1 + my) * 2 * mx];
            }
            a[ix] = mkc<double>(v0, v1);
        }
        double2 *z = line_fft<double>(a, b, cv.px, cv.twx, -1, lane, nl, L.blk);
        for (int k = lane; k < nkx; k += nl) {
            double2 zk = z[k], zn = z[(NX - k) % NX];
            S[(size_t)k * NY + r0] = mkc<double>(0.5 * (zk.x + zn.x), 0.5 * (zk.y - zn.y));
            S[(size_t)k * NY + r1] = mkc<double>(0.5 * (zk.y + zn.y), 0.5 * (zn.x - zk.x));
        }
        line_sync(L.blk);
    }
    gsync();
    for (int kx = L.w0; kx < nkx; kx += L.nw) {
        for (int iy = lane; iy < NY; iy += nl) a[iy] = S[(size_t)kx * NY + iy];
        double2 *z = line_fft<double>(a, b, cv.py, cv.twy, -1, lane, nl, L.blk);
        for (int ky = lane; ky <= fy; ky += nl) {
            const size_t o = (size_t)kx * (fy + 1) + ky;
            const double v = imag ? z[ky].y : z[ky].x;
            K64[o] = v;
            K32[o] = (float)v;
        }
        line_sync(L.blk);
    }
    gsync();
}

// preconditioner kernel m = ga^2 IFFT(1 ./ FFT(c)) / (P Q) over the period P = 2mx, Q = 2my
// (fft_makePrec, src/m_aijpj.f90:457-708), written in the layout of cf.  S: P*Q complex.
__device__ __noinline__ void prec_spatial(const Lines &L, const double *src, int mx, int my, double ga,
                                          const FftPlan &pp, const FftPlan &pq, const double2 *twp,
                                          const double2 *twq, double2 *S, double *dst, double2 *a, double2 *b) {
    const int P = 2 * mx, Q = 2 * my;
    const int lane = L.lane, nl = L.nl;
    gsync();
    for (int iy = L.w0; iy < Q; iy += L.nw) {
        const int dy = iy < my ? iy : iy - Q;
        for (int ix = lane; ix < P; ix += nl) {
            const int dx = ix < mx ? ix : ix - P;
            a[ix] = mkc<double>(src[(size_t)(dx + mx) + (size_t)(dy + my) * 2 * mx], 0.0);
        }
        double2 *z = line_fft<double>(a, b, pp, twp, -1, lane, nl, L.blk);
        for (int k = lane; k < P; k += nl) S[(size_t)iy * P + k] = z[k];
        line_sync(L.blk);
    }
    gsync();
    const double g2 = ga * ga;
    for (int kx = L.w0; kx < P; kx += L.nw) {
        for (int iy = lane; iy < Q; iy += nl) a[iy] = S[(size_t)iy * P + kx];
        double2 *z = line_fft<double>(a, b, pq, twq, -1, lane, nl, L.blk);
        for (int ky = lane; ky < Q; ky += nl) {
            const double2 c = z[ky];
            const double den = c.x * c.x + c.y * c.y;
            z[ky] = mkc<double>(g2 * c.x / den, -g2 * c.y / den);
        }
        line_sync(L.blk);
        double2 *o = (z == a) ? b : a;
        double2 *r = line_fft<double>(z, o, pq, twq, +1, lane, nl, L.blk);
        for (int iy = lane; iy < Q; iy += nl) S[(size_t)iy * P + kx] = r[iy];
        line_sync(L.blk);
    }
    gsync();
    const double sc = 1.0 / ((double)P * (double)Q);
    for (int iy = L.w0; iy < Q; iy += L.nw) {
        const int dy = iy < my ? iy : iy - Q;
        for (int ix = lane; ix < P; ix += nl) a[ix] = S[(size_t)iy * P + ix];
        double2 *z = line_fft<double>(a, b, pp, twp, +1, lane, nl, L.blk);
        for (int ix = lane; ix < P; ix += nl) {
            const int dx = ix < mx ? ix : ix - P;
            dst[(size_t)(dx + mx) + (size_t)(dy + my) * 2 * mx] = z[ix].x * sc;
        }
        line_sync(L.blk);
    }
    gsync();
}

// grid: one CTA per listed patch (group == 0), or the nblk CTAs of one patch group (group
// != 0, cooperative launch, list[0] is the patch)
__global__ void __launch_bounds__(kThreads) k_spectra(const PatchDesc *descs, const int *list, int group) {
    extern __shared__ __align__(16) unsigned char smraw[];
    const PatchDesc &d = descs[list[group ? 0 : blockIdx.x]];
    const bool blk = group != 0;
    group_init(blk ? d.nblk : 1, blk ? (int)blockIdx.x : 0, d.gscr);
    const SmemPlan sp = smem_plan(d.fx, d.fy, blk);
    Conv<double> cv = make_conv<double>(d, smraw, sp);
    // one line at a time per CTA (all its threads on the line): the batch buffer holds one
    // CTA-wide line region of 4 nmax complex
    cv.L = line_workers(true);
    const int mx = d.mx, my = d.my;
    const size_t bsz = (size_t)4 * mx * my;
    const size_t ksz = (size_t)cv.nkx * (d.fy + 1);
    double *K64 = const_cast<double *>(d.spec64);
    float *K32 = const_cast<float *>(d.spec32);
    double2 *a = cv.wbuf + cv.L.widx * cv.wstride, *b = a + 2 * sp.nmax;
    // scratch in the work columns: S (complex), then the spatial preconditioner kernel
    double2 *S = (double2 *)d.wk;
    const size_t s_dbl = spectra_scratch_doubles(mx, my, d.fx, d.fy);
    double *msp = d.wk + s_dbl;
    // twiddles of the preconditioner period: shared memory (single CTA, reusing the
    // convolution tables) or their own tables in the group scratch
    double2 *twpx = cv.twx, *twpy = cv.twy;
    if (blk) {
        const GroupTw g = group_tw(d.nblk, mx, my, d.fx, d.fy);
        twpx = (double2 *)((char *)d.gscr + g.offpx);
        twpy = (double2 *)((char *)d.gscr + g.offpy);
        make_twiddles<double>(cv.twx, cv.NX, true);
        make_twiddles<double>(cv.twy, cv.NY, true);
        make_twiddles<double>(twpx, 2 * mx, true);
        make_twiddles<double>(twpy, 2 * my, true);
    }
    for (int blkc = 0; blkc < 4; blkc++) {
        if (!blk) {
            make_twiddles<double>(cv.twx, cv.NX);
            make_twiddles<double>(cv.twy, cv.NY);
        }
        block_spectrum(cv, d.cf + blkc * bsz, S, K64 + blkc * ksz, K32 + blkc * ksz, a, b);
    }
    // preconditioners zz -> 4, xx -> 5, yy -> 6
    FftPlan pp, pq;
    fft_factorize(2 * mx, pp);
    fft_factorize(2 * my, pq);
    const int srcblk[3] = {3, 0, 2};
    for (int k = 0; k < 3; k++) {
        gsync();
        if (!blk) {
            make_twiddles<double>(twpx, 2 * mx);
            make_twiddles<double>(twpy, 2 * my);
        }
        prec_spatial(cv.L, d.cf + srcblk[k] * bsz, mx, my, d.ga, pp, pq, twpx, twpy, S, msp, a, b);
        if (!blk) {
            make_twiddles<double>(cv.twx, cv.NX);
            make_twiddles<double>(cv.twy, cv.NY);
        }
        block_spectrum(cv, msp, S, K64 + (4 + k) * ksz, K32 + (4 + k) * ksz, a, b);
    }
    // coupling blocks (K != 0): xz, yz (odd in x, resp. y: imaginary spectra) -> spectra 7, 8;
    // in steady rolling xz, yz of cs - cv (no parity in x: real and imaginary parts) -> 9, 10
    // and 11, 12
    for (int q = 0; q < spectra_count(d.ncf) - 7; q++) {
        const int blkc = q < 2 ? 4 + q : 6 + (q - 2) / 2;
        const bool im = q < 2 ? true : ((q - 2) % 2 == 1);
        gsync();
        if (!blk) {
            make_twiddles<double>(cv.twx, cv.NX);
            make_twiddles<double>(cv.twy, cv.NY);
        }
        block_spectrum(cv, d.cf + blkc * bsz, S, K64 + (7 + q) * ksz, K32 + (7 + q) * ksz, a, b, im);
    }
}

// ------------------------------------------------------------------------------------------
// set-up: right-hand sides (set_norm_rhs / set_tang_rhs, m_sdis.f90:321-583) and initial
// estimate (init_curr_data / eldiv0, m_sdis.f90:587-1009)
// ------------------------------------------------------------------------------------------
__device__ __noinline__ void setup_patch(const PView &P) {
    const PatchDesc &d = *P.d;
    const int mx = P.mx, n = P.n;
    RedSmem &red = P.sm->red;
    int *igs = P.igs();
    double *h = P.c(W_H), *wx = P.c(W_WX), *wy = P.c(W_WY);
    double *px = P.c(W_PX), *py = P.c(W_PY), *pn = P.c(W_PN);
    const bool is_roll = d.tang == 2 || d.tang == 3;
    const double facphi = 1.0 / 6.0;
    const double xofs = is_roll ? cos(d.chi) * d.dq * facphi : 0.0;
    const double yofs = is_roll ? sin(d.chi) * d.dq * facphi : 0.0;
    // initial estimate from the problem's previous solution kept in device memory, regularised
    // as init_curr_data does (m_sdis.f90:716-729): I = 1 zeroes exterior tractions and puts slip
    // tractions on the bound, I = 2 keeps the contact area only
    if (d.prev && d.iestim != 0) {
        const double *qx = d.prev, *qy = d.prev + n, *qn = d.prev + 2 * (size_t)n;
        const int *qg = (const int *)(d.prev + 3 * (size_t)n);
        FOR_I(ii, n) {
            int g = qg[ii];
            double ax = qx[ii], ay = qy[ii], an = qn[ii];
            if (d.iestim == 1) {
                if (g <= Exter) { an = ax = ay = 0.0; }
                else if (g == Slip) {
                    const double pabs = fmax(1e-10, sqrt(ax * ax + ay * ay));
                    ax = d.fstat * an * ax / pabs;
                    ay = d.fstat * an * ay / pabs;
                }
            }
            if (d.iestim == 2) { if (g >= Adhes) g = Adhes; ax = ay = 0.0; }
            igs[ii] = g; px[ii] = ax; py[ii] = ay; pn[ii] = an;
        }
        gsync();
    }
    FOR_I(ii, n) {
        const double x = d.xc1 + (ii % mx) * d.dx, y = d.yc1 + (ii / mx) * d.dy;
        if (d.ibase != 9) h[ii] = d.prm[0] * x * x + d.prm[1] * x * y + d.prm[2] * y * y + d.prm[3] * x + d.prm[4] * y + d.prm[5];
        double vx = -(y + yofs) * d.cphi, vy = (x + xofs) * d.cphi;
        if (d.force3 == 0) vx += d.cksi;
        if (d.force3 <= 1) vy += d.ceta;
        wx[ii] = -d.dq * vx;
        wy[ii] = -d.dq * vy;
        if (d.iestim == 0) { pn[ii] = 0.0; igs[ii] = Exter; }
        if (d.iestim == 0 || d.iestim == 2 || d.tang == 0) { px[ii] = 0.0; py[ii] = 0.0; }
    }
    gsync();
    const bool use_hz = (d.iestim == 0 && d.bound == 0 && d.ihertz >= 1);
    const double pi = 3.14159265358979323846;
    if ((d.bound == 2 || use_hz) && d.ihertz <= 3) {
        const double pnmax = 3.0 * d.fntrue / (2.0 * pi * d.aa * d.bb);
        FOR_I(ii, n) {
            const double x = d.xc1 + (ii % mx) * d.dx, y = d.yc1 + (ii / mx) * d.dy;
            const double f = 1.0 - (x / d.aa) * (x / d.aa) - (y / d.bb) * (y / d.bb);
            pn[ii] = pnmax * sqrt(fmax(0.0, f));
        }
    }
    if (d.bound == 3 && d.ihertz <= 3) {
        const double pnmax = 2.0 * d.fntrue / (pi * d.aa * d.bb);
        FOR_I(ii, n) {
            const double x = d.xc1 + (ii % mx) * d.dx, y = d.yc1 + (ii / mx) * d.dy;
            const double f = 1.0 - (x / d.aa) * (x / d.aa) - (y / d.bb) * (y / d.bb);
            pn[ii] = pnmax * fmax(0.0, f);
        }
    }
    gsync();
    if ((d.bound >= 2 && d.bound <= 4) || use_hz) {
        FOR_I(ii, n) igs[ii] = (pn[ii] > (double)1e-20f) ? Adhes : Exter;
    } else if (d.iestim == 0) {
        double hmin = 1e300; FOR_I(ii, n) hmin = fmin(hmin, h[ii]);
        hmin = block_min1(red, hmin);
        double pentru = d.pen - hmin;
        const double facpen = (double)0.60f, reltol = (double)0.01f;
        if (d.norm == 1 && d.my > 1) {
            const double fnscal = d.fntrue / d.ga;
            const double fac = 1.0 * 0.75 * sqrt(pi) * (1.0 - d.nu);
            double penmin = 0.0, fnmin = 0.0;
            double penmax = fac * fnscal / sqrt(d.dxdy);
            int c = 0; FOR_I(ii, n) if (h[ii] - hmin < facpen * penmax) c++;
            c = block_sumi1(red, c);
            double fnmax = penmax * sqrt(d.dxdy * c) / fac;
            int iter = 0;
            while (iter < 50 && fabs(fnmax - fnmin) > reltol * fnscal) {
                iter++;
                double penmid = 0.5 * (penmax + penmin);
                int cm = 0; FOR_I(ii, n) if (h[ii] - hmin < facpen * penmid) cm++;
                cm = block_sumi1(red, cm);
                double fnmid = penmid * sqrt(d.dxdy * cm) / fac;
                if (fnmid < fnscal) { penmin = penmid; fnmin = fnmid; }
                else { penmax = penmid; fnmax = fnmid; }
            }
            pentru = penmax;
        }
        FOR_I(ii, n) igs[ii] = (h[ii] - hmin < facpen * pentru) ? Adhes : Exter;
    }
    gsync();
    FOR_I(ii, n) if (h[ii] > (double)1e29f) igs[ii] = Exter;
    gsync();
}

// leading-edge fraction facdt (sxbnd, m_leadedge.f90:92-332) for rolling direction chi = 0.
// edge (optional, ConvexGS in steady rolling): per element the 1-based column of its leading
// edge where the element lies within one rolling step of it (facdt < 0.9999, the reference's
// ii2j > 0), else 0
__device__ __noinline__ void compute_facdt(const PView &P, int solver, double *facdt, int *edge = nullptr) {
    const PatchDesc &d = *P.d;
    const int mx = P.mx, my = P.my;
    const int *igs = P.igs();
    const bool is_roll = d.tang == 2 || d.tang == 3;
    const double fxdfac = (solver == 4) ? 2.0 : 1.0;
    gsync();
    FOR_ROW(iy, my) {
        const int i0 = iy * mx;
        int ixb = mx;
        for (int ix = mx; ix >= 1; ix--) {
            const int ii = (ix - 1) + i0;
            if ((igs[ii] >= Adhes) && (ix == mx || igs[ii + 1] <= Exter)) ixb = ix;
            int je = 0;
            if (!is_roll) facdt[ii] = 1.0;
            else if (igs[ii] <= Exter) facdt[ii] = 0.0;
            else if (ix + 2 > mx) facdt[ii] = 1.0;
            else {
                const double xbnd = d.xc1 + (ixb - 1) * d.dx + fxdfac * d.dx;
                const double x = d.xc1 + (ix - 1) * d.dx;
                facdt[ii] = fmin(1.0, (xbnd - x) / d.dq);
                if (facdt[ii] < 0.9999) je = ixb;
            }
            if (edge) edge[ii] = je;
        }
    }
    gsync();
}


// state of TANG shared by the solver dispatch and the Newton-Raphson on total forces
struct TangRun {
    int solver;
    double omegah, omegas, eps, eps32;
    const Ops<double> *op;
    const Ops<float> *o32;
    const double *csv;            // ConvexGS in steady rolling: csv = cs - cv
    const int *edge;              // ConvexGS: leading-edge column per element
    bool any_edge, gs_ok;
    int nconv, nconv32, nls;
    double fntrue;                // total normal force of the solution
    double cksi, ceta;            // creepages (updated when total forces are prescribed)
    double *sens;                 // sensitivities [out * 4 + in]: out Fn, Fx, Fy, Mz; in pen, cksi, ceta, cphi
    int maxgs;                    // iterations and tolerance of the current solve (the sensitivity
    const double *p0x, *p0y;      // solves change them); p0: base of their stopping rule
};

// tang_solver, m_solvpt.f90:382-493: one solve of the tangential problem for the current element
// division and shift ws (W_WSX, W_WSY).  Returns the iterations; -1000 for a Gauss-Seidel solver
// on a patch group too large for it, -2000 on a failed line search.
__device__ __noinline__ int tang_solver(const PView &P, TangRun &T, int &info, double &errpt) {
    const PatchDesc &d = *P.d;
    int it = 0;
    info = 0;
    errpt = 0.0;
    const int maxgs = T.maxgs;
    if (T.solver == 4) {
        it = stdygs(P, T.eps, maxgs, T.omegah, T.omegas, info, errpt, T.o32 ? T.op : nullptr, T.p0x, T.p0y);
    } else if (T.solver == 3) {
        it = cnvxgs(P, *T.op, T.csv, T.edge, T.any_edge, T.eps, maxgs, T.omegah, T.omegas, info, errpt, T.p0x, T.p0y);
    } else if (T.solver == 7) {
        bool lstagn = false;
        it = gdsteady<double>(P, *T.op, maxgs, T.eps, errpt, lstagn, T.nconv, T.nls, T.o32, T.nconv32);
        if (it == -100000) return -2000;
        if (lstagn && !T.gs_ok) return -1000;
        if (lstagn)
            it = stdygs(P, T.eps, maxgs, T.omegah, T.omegas, info, errpt, T.o32 ? T.op : nullptr, T.p0x, T.p0y);
    } else {
        int it32 = 0;
        if (T.o32) {
            it32 = tangcg<float>(P, *T.o32, T.o32->K[5], T.o32->K[6], maxgs, fmax(T.eps32, T.eps), errpt, T.nconv32,
                                 T.p0x, T.p0y);
            it32 = it32 > 0 ? it32 : 0;
        }
        it = tangcg<double>(P, *T.op, T.op->K[5], T.op->K[6], maxgs, T.eps, errpt, T.nconv, T.p0x, T.p0y) + it32;
    }
    return it;
}

// total tangential forces relative to mu Fn
__device__ inline void rel_forces(const PView &P, const TangRun &T, double &fx, double &fy) {
    const PatchDesc &d = *P.d;
    const double *px = P.c(W_PX), *py = P.c(W_PY);
    double a[2] = {0.0, 0.0};
    FOR_I(i, P.n) { a[0] += px[i]; a[1] += py[i]; }
    block_sum<2>(P.sm->red, a);
    fx = d.dxdy * a[0] / (d.fstat * T.fntrue);
    fy = d.dxdy * a[1] / (d.fstat * T.fntrue);
}

// solvpt, m_solvpt.f90:51-378: the tangential solve with shift wstot = wsfix + facdt dq (cksi,
// ceta) for the prescribed components; with total forces prescribed (F=1: Fx, F=2: Fx and Fy) a
// Newton-Raphson iteration on cksi (and ceta) around it, its derivatives the secants of its own
// steps.  Returns the solver iterations summed over the Newton-Raphson steps (negative codes as
// tang_solver); errpt includes the Newton-Raphson residual as the reference adds it.
__device__ __noinline__ int solvpt(const PView &P, TangRun &T, int &info, double &errpt) {
    const PatchDesc &d = *P.d;
    const int n = P.n, f3 = d.force3;
    const int *iel = P.ci(I_IEL);
    const double *facdt = P.c(W_FACDT), *wfx = P.c(W_WFX), *wfy = P.c(W_WFY);
    double *wsx = P.c(W_WSX), *wsy = P.c(W_WSY);
    const double dq = d.dq;
    FOR_I(i, n) {
        wsx[i] = wfx[i];
        wsy[i] = wfy[i];
        if (iel[i] && f3 >= 1) wsx[i] += facdt[i] * T.cksi * dq;
        if (iel[i] && f3 >= 2) wsy[i] += facdt[i] * T.ceta * dq;
    }
    gsync();
    int it = tang_solver(P, T, info, errpt);
    if (it < 0 || f3 == 0) return it;
    int itgs = it;
    double fxkp1, fykp1;
    rel_forces(P, T, fxkp1, fykp1);
    // the Newton-Raphson's secants dFx/dcksi, dFy/dcksi, dFx/deta, dFy/deta
    double &s_xk = T.sens[1 * 4 + 1], &s_yk = T.sens[2 * 4 + 1], &s_xe = T.sens[1 * 4 + 2], &s_ye = T.sens[2 * 4 + 2];
    double sens[4] = {s_xk, s_yk, s_xe, s_ye};
    if (info <= 1) {
        int itnr = 0;
        double df = fabs(d.fxrel - fxkp1);
        if (f3 >= 2) df += fabs(d.fyrel - fykp1);
        int nadh = 0, nslip = 0, nplast = 0, nexter = 0;
        count_eldiv(P, nadh, nslip, nplast, nexter);
        while (df > T.eps && itnr < d.maxnr && info <= 1) {
            itnr++;
            const double dfx = d.fxrel - fxkp1, dfy = d.fyrel - fykp1;
            double dcksi = 0.0, dceta = 0.0;
            if (f3 == 1) {
                if (fabs(sens[0]) > (double)1e-6f) dcksi = dfx / sens[0];
                else dcksi = (double)0.00003f;
            } else {
                const double det = sens[0] * sens[3] - sens[1] * sens[2];
                if (det > T.eps) {
                    dcksi = (sens[3] * dfx - sens[1] * dfy) / det;
                    dceta = (-sens[2] * dfx + sens[0] * dfy) / det;
                } else {
                    dcksi = 0.000003;
                    dceta = 0.000003;
                }
            }
            for (int ifxy = 1; ifxy <= f3; ifxy++) {
                const double fxk = fxkp1, fyk = fykp1;
                const double dc = ifxy == 1 ? dcksi : dceta;
                if (ifxy == 1) T.cksi += dcksi; else T.ceta += dceta;
                double *w = ifxy == 1 ? wsx : wsy;
                FOR_I(i, n) if (iel[i]) w[i] += facdt[i] * dc * dq;
                gsync();
                it = tang_solver(P, T, info, errpt);
                if (it < 0) return it;
                itgs += it;
                rel_forces(P, T, fxkp1, fykp1);
                count_eldiv(P, nadh, nslip, nplast, nexter);
                const double dfxk = fxkp1 - fxk, dfyk = fykp1 - fyk;
                const double scl = d.fstat * T.fntrue / ((nadh + nslip + nplast) * d.dxdy);
                if (ifxy == 1) {
                    if (nadh > 0) {
                        if (sens[0] == 0.0 || fabs(dfxk * scl) > 10.0 * errpt) sens[0] = dfxk / dcksi;
                        if (fabs(dfyk * scl) > 10.0 * errpt) sens[1] = dfyk / dcksi;
                    } else if (fabs(sens[0]) < (double)1e-6f) {
                        sens[0] = fxkp1 / T.cksi;
                    }
                } else {
                    if (nadh > 0) {
                        if (fabs(dfxk * scl) > 10.0 * errpt) sens[2] = dfxk / dceta;
                        if (sens[3] == 0.0 || fabs(dfyk * scl) > 10.0 * errpt) sens[3] = dfyk / dceta;
                    } else if (fabs(sens[3]) < (double)1e-6f) {
                        sens[3] = fykp1 / T.ceta;
                    }
                }
                df = fabs(d.fxrel - fxkp1);
                if (f3 >= 2) df += fabs(d.fyrel - fykp1);
            }
        }
        // the Newton-Raphson residual joins the error estimate, with the element code Slip (= 2)
        // in the place of the number of slip elements as in the reference (m_solvpt.f90:361)
        errpt += 2.0 * df * d.fstat * T.fntrue / ((nadh + Slip + nplast) * d.dxdy);
    } else {
        sens[0] = sens[1] = sens[2] = sens[3] = 0.0;
    }
    s_xk = sens[0]; s_yk = sens[1]; s_xe = sens[2]; s_ye = sens[3];
    return itgs;
}

// Kalker's coefficients of the linear theory for an elliptic contact: C11, C22, C23 at nu = 0,
// 1/4, 1/2 for g = min(a/b, b/a) = 0.1 .. 1 (Kalker 1990, table E.3), as single-precision values
// like the reference's data statement (linrol, m_hertz.f90:1147-1247).  [a < b | a > b][g row]
// [C11, C22, C23][nu].  Published theory: the values are the table's.
__constant__ float c_kalker[2][10][3][3] = {
    {{{2.51f, 3.31f, 4.85f}, {2.51f, 2.52f, 2.53f}, {.334f, .473f, .731f}},
     {{2.59f, 3.37f, 4.81f}, {2.59f, 2.63f, 2.66f}, {.483f, .603f, .809f}},
     {{2.68f, 3.44f, 4.80f}, {2.68f, 2.75f, 2.81f}, {.607f, .715f, .889f}},
     {{2.78f, 3.53f, 4.82f}, {2.78f, 2.88f, 2.98f}, {.720f, .823f, .977f}},
     {{2.88f, 3.62f, 4.83f}, {2.88f, 3.01f, 3.14f}, {.827f, .929f, 1.07f}},
     {{2.98f, 3.72f, 4.91f}, {2.98f, 3.14f, 3.31f}, {.930f, 1.03f, 1.18f}},
     {{3.09f, 3.81f, 4.97f}, {3.09f, 3.28f, 3.48f}, {1.03f, 1.14f, 1.29f}},
     {{3.19f, 3.91f, 5.05f}, {3.19f, 3.41f, 3.65f}, {1.13f, 1.25f, 1.40f}},
     {{3.29f, 4.01f, 5.12f}, {3.29f, 3.54f, 3.82f}, {1.23f, 1.36f, 1.51f}},
     {{3.40f, 4.12f, 5.20f}, {3.40f, 3.67f, 3.98f}, {1.33f, 1.47f, 1.63f}}},
    {{{10.7f, 11.7f, 12.9f}, {10.7f, 12.8f, 16.0f}, {12.2f, 14.6f, 18.0f}},
     {{6.96f, 7.78f, 8.82f}, {6.96f, 8.14f, 9.79f}, {5.72f, 6.63f, 7.89f}},
     {{5.57f, 6.34f, 7.34f}, {5.57f, 6.40f, 7.51f}, {3.79f, 4.32f, 5.01f}},
     {{4.84f, 5.57f, 6.57f}, {4.84f, 5.48f, 6.31f}, {2.88f, 3.24f, 3.70f}},
     {{4.37f, 5.10f, 6.11f}, {4.37f, 4.90f, 5.56f}, {2.35f, 2.62f, 2.96f}},
     {{4.06f, 4.78f, 5.80f}, {4.06f, 4.50f, 5.04f}, {2.01f, 2.23f, 2.50f}},
     {{3.82f, 4.54f, 5.58f}, {3.82f, 4.21f, 4.67f}, {1.76f, 1.95f, 2.18f}},
     {{3.65f, 4.36f, 5.42f}, {3.65f, 3.99f, 4.39f}, {1.58f, 1.75f, 1.94f}},
     {{3.51f, 4.22f, 5.30f}, {3.51f, 3.81f, 4.16f}, {1.44f, 1.59f, 1.77f}},
     {{3.40f, 4.12f, 5.20f}, {3.40f, 3.67f, 3.98f}, {1.33f, 1.47f, 1.63f}}}};

// creepage coefficients C11, C22, C23 of the linear theory for Poisson's ratio nu and semi-axes
// ratio aob: interpolation in the table, the asymptotes of slender ellipses (g < 0.1)
__device__ void linrol(double nu, double aob, double &cxx, double &cyy, double &cyz) {
    const double pi = 3.14159265358979323846;
    int icase;
    double g;
    if (aob <= 1.0) { g = aob; icase = 0; } else { g = 1.0 / aob; icase = 1; }
    if (icase == 0 && g < 0.101) {
        cxx = pi * pi / 4.0 / (1.0 - nu);
        cyy = pi * pi / 4.0;
        cyz = pi * sqrt(g) / 3.0 / (1.0 - nu) * (1.0 + nu * (log(16.0 / g) - 5.0));
    } else if (icase == 1 && g < 0.101) {
        const double al = log(16.0 / (g * g));
        cxx = 2.0 * pi / (al - 2.0 * nu) / g * (1.0 + (3.0 - log(4.0)) / (al - 2.0 * nu));
        cyy = 2.0 * pi / g * (1.0 + (1.0 - nu) * (3.0 - log(4.0)) / ((1.0 - nu) * al + 2.0 * nu)) /
              ((1.0 - nu) * al + 2.0 * nu);
        cyz = 2.0 * pi / 3.0 / pow(g, 1.5) / ((1.0 - nu) * al - 2.0 + 4.0 * nu);
    } else {
        const int irow = (int)(10.0 * g - 0.005);
        const double fac = 10.0 * g - (double)(float)irow;
        double cc[3];
        for (int ic = 0; ic < 3; ic++) {
            double cn[3];
            for (int in = 0; in < 3; in++)
                cn[in] = fac * (double)c_kalker[icase][irow][ic][in] + (1.0 - fac) * (double)c_kalker[icase][irow - 1][ic][in];
            cc[ic] = (nu - 0.25) * (nu - 0.50) * 8.0 / cn[0] - (nu - 0.50) * nu * 16.0 / cn[1] +
                     nu * (nu - 0.25) * 8.0 / cn[2];
        }
        cxx = 1.0 / cc[0]; cyy = 1.0 / cc[1]; cyz = 1.0 / cc[2];
    }
}

// char_creep, m_solvpt.f90:497-540: characteristic creepages of the linear theory, with the
// contact's radius from its area and its semi-axes from the bounding box of its elements
__device__ __noinline__ void char_creep(const PView &P, double fntrue, double ch[3]) {
    const PatchDesc &d = *P.d;
    const int mx = P.mx, n = P.n;
    const int *igs = P.igs();
    int c = 0, ix0 = mx + 1, ix1 = 0, iy0 = P.my + 1, iy1 = 0;
    FOR_I(i, n) if (igs[i] >= Adhes) {
        c++;
        const int ix = i % mx + 1, iy = i / mx + 1;
        ix0 = min(ix0, ix); ix1 = max(ix1, ix); iy0 = min(iy0, iy); iy1 = max(iy1, iy);
    }
    RedSmem &red = P.sm->red;
    c = block_sumi1(red, c);
    ix0 = (int)block_min1(red, (double)ix0); ix1 = (int)block_max1(red, (double)ix1);
    iy0 = (int)block_min1(red, (double)iy0); iy1 = (int)block_max1(red, (double)iy1);
    if (c == 0) { ix0 = mx; ix1 = 1; iy0 = P.my; iy1 = 1; }
    const double pi = 3.14159265358979323846;
    const double rc = sqrt((double)(float)c * d.dx * d.dy / pi);
    const double a = (double)(float)max(1, ix1 - ix0 + 1) * d.dx * 0.5;
    const double b = (double)(float)max(1, iy1 - iy0 + 1) * d.dy * 0.5;
    double c11, c22, c23;
    linrol(d.nu, a / b, c11, c22, c23);
    ch[0] = d.fstat * fntrue / (rc * rc * d.ga * c11);
    ch[1] = d.fstat * fntrue / (rc * rc * d.ga * c22);
    ch[2] = d.fstat * fntrue / (rc * rc * rc * d.ga * c23);
}

// Mz of the current tangential tractions
__device__ inline double moment_z(const PView &P) {
    const PatchDesc &d = *P.d;
    const double *px = P.c(W_PX), *py = P.c(W_PY);
    double a[2] = {0.0, 0.0};
    FOR_I(i, P.n) {
        const double x = d.xc1 + (i % P.mx) * d.dx, y = d.yc1 + (i / P.mx) * d.dy;
        a[0] += px[i] * y; a[1] += py[i] * x;
    }
    block_sum<2>(P.sm->red, a);
    return d.dxdy * (-a[0] + a[1]);
}

// sens_norm, m_solvpn.f90:531-650: d Fn / d pen from one NormCG solve with the approach raised by
// 0.67 % of the largest normal displacement in contact, started from the solution (which is
// restored afterwards), with the stopping rule on the change from that start.  unn: the normal
// displacements of the solution (W_DD).  False when that solve diverges.
__device__ __noinline__ bool sens_norm(const PView &P, const Ops<double> &op, double pen, double fntrue, int &nconv,
                                       double &sens_fn_pen) {
    const PatchDesc &d = *P.d;
    const int n = P.n;
    RedSmem &red = P.sm->red;
    int *igs = P.igs();
    double *pn = P.c(W_PN), *pn0 = P.c(W_RX), *ig0 = P.c(W_RY);
    const double *unn = P.c(W_DD);
    double m = -1e300;
    FOR_I(i, n) { if (igs[i] >= Adhes) m = fmax(m, unn[i]); pn0[i] = pn[i]; ig0[i] = (double)igs[i]; }
    const double pentru = block_max1(red, m);
    const double dpen = 0.0067 * pentru;
    double penloc = pen + dpen, err = 0.0;
    const int it = normcg<double>(P, op, d.mxsens, d.epsens, penloc, err, nconv, 0, pn0);
    double s = 0.0;
    FOR_I(i, n) s += pn[i];
    const double fnloc = d.dxdy * block_sum1(red, s);
    sens_fn_pen = (fnloc - fntrue) / dpen;
    FOR_I(i, n) { pn[i] = pn0[i]; igs[i] = (int)ig0[i]; }
    gsync();
    return it >= 0;
}

// sens_tang, m_solvpt.f90:544-796: d(Fx, Fy, Mz) / d(cksi, ceta, cphi) from one extra tangential
// solve per creepage, perturbed by 1e-4 of its characteristic size and started from the solution
// (restored afterwards), with the sensitivity solves' iterations, tolerance and stopping rule.
// Returns false when a solve failed.
__device__ __noinline__ bool sens_tang(const PView &P, TangRun &T) {
    const PatchDesc &d = *P.d;
    const int n = P.n, mx = P.mx, f3 = d.force3;
    int *igs = P.igs();
    const int *iel = P.ci(I_IEL);
    double *px = P.c(W_PX), *py = P.c(W_PY), *sx = P.c(W_SX), *sy = P.c(W_SY);
    double *wsx = P.c(W_WSX), *wsy = P.c(W_WSY);
    const double *wfx = P.c(W_WFX), *wfy = P.c(W_WFY), *facdt = P.c(W_FACDT);
    double *px0 = P.c(W_RES), *py0 = P.c(W_RPRV), *sx0 = P.c(W_Z), *sy0 = P.c(W_V), *ig0 = P.c(W_Q);
    double fxrel, fyrel;
    rel_forces(P, T, fxrel, fyrel);
    const double mztrue = moment_z(P);
    double ch[3];
    char_creep(P, T.fntrue, ch);
    FOR_I(i, n) { px0[i] = px[i]; py0[i] = py[i]; sx0[i] = sx[i]; sy0[i] = sy[i]; ig0[i] = (double)igs[i]; }
    gsync();
    const int maxgs0 = T.maxgs;
    const double eps0 = T.eps;
    bool ok = true;
    for (int icrp = 1; icrp <= 3 && ok; icrp++) {
        const double dcrp = 0.0001 * ch[icrp - 1];
        FOR_I(i, n) {
            double wx = wfx[i], wy = wfy[i];
            if (iel[i]) {
                if (f3 >= 1) wx += facdt[i] * T.cksi * d.dq;
                if (f3 >= 2) wy += facdt[i] * T.ceta * d.dq;
                if (icrp == 1) wx += facdt[i] * dcrp * d.dq;
                else if (icrp == 2) wy += facdt[i] * dcrp * d.dq;
                else {
                    const double x = d.xc1 + (i % mx) * d.dx, y = d.yc1 + (i / mx) * d.dy;
                    wx -= facdt[i] * dcrp * y * d.dq;
                    wy += facdt[i] * dcrp * x * d.dq;
                }
            }
            wsx[i] = wx; wsy[i] = wy;
        }
        gsync();
        T.maxgs = d.mxsens; T.eps = d.epsens; T.p0x = px0; T.p0y = py0;
        int info = 0;
        double err = 0.0;
        const int it = tang_solver(P, T, info, err);
        T.maxgs = maxgs0; T.eps = eps0; T.p0x = nullptr; T.p0y = nullptr;
        if (it < 0) ok = false;
        double fxloc, fyloc;
        rel_forces(P, T, fxloc, fyloc);
        const double mzloc = moment_z(P);
        T.sens[1 * 4 + icrp] = (fxloc - fxrel) / dcrp;
        T.sens[2 * 4 + icrp] = (fyloc - fyrel) / dcrp;
        T.sens[3 * 4 + icrp] = (mzloc - mztrue) / dcrp;
        FOR_I(i, n) { px[i] = px0[i]; py[i] = py0[i]; sx[i] = sx0[i]; sy[i] = sy0[i]; igs[i] = (int)ig0[i]; }
        gsync();
    }
    return ok;
}

// TANG, m_stang.f90:28-746 for Coulomb friction, creepages or total forces prescribed.
// Returns ittang; -1000 for a Gauss-Seidel solver on a patch group too large for it, -2000 on
// a failed line search.  With T.o32 (mixed precision): GDsteady runs once with FP32 direction
// products and FP64 residual replacement; SteadyGS takes FP32 sums of its in-sweep changes on
// an FP64 base; TangCG runs an FP32 pass to eps32 followed by an FP64 pass.
__device__ __noinline__ int stang(const PView &P, TangRun &T, int &itgs_out) {
    const PatchDesc &d = *P.d;
    const int mx = P.mx, my = P.my, n = P.n;
    RedSmem &red = P.sm->red;
    int *igs = P.igs(), *iel = P.ci(I_IEL);
    const bool is_ssrol = d.tang == 3;
    double *px = P.c(W_PX), *py = P.c(W_PY), *pn = P.c(W_PN), *sx = P.c(W_SX), *sy = P.c(W_SY);
    double *wfx = P.c(W_WFX), *wfy = P.c(W_WFY), *wx = P.c(W_WX), *wy = P.c(W_WY);
    int nadh, nslip, nplast, nexter;
    count_eldiv(P, nadh, nslip, nplast, nexter);
    const int k = nadh + nslip + nplast;
    int icount = 0;
    FOR_ROW(iy, my) if (igs[iy * mx] >= Adhes) icount++;
    icount = block_sumi1(red, icount);
    int solver;
    if (is_ssrol) solver = (d.gausei == 5) ? 7 : (d.gausei != 2 ? 4 : 3);
    else solver = (d.gausei != 2) ? 2 : 3;
    if (icount > 0 && (solver == 4 || solver == 7)) solver = 3;
    double omegah = d.omegah, omegas = d.omegas;
    if (d.gausei == 0 || d.gausei == 4 || d.gausei == 5) {
        if (k <= 25) { omegah = 1.0; omegas = 1.0; }
        else if (is_ssrol && solver == 3) { omegah = 0.5; omegas = 0.5; }
        else if (is_ssrol) {
            if (d.dx / d.dy <= 5.0) { omegah = 0.9; omegas = 1.0; }
            else if (d.dx / d.dy <= 15.0) { omegah = 0.8; omegas = 0.8; }
            else { omegah = 0.8; omegas = 0.6; }
        } else { omegah = 0.5; omegas = 0.5; }
    }
    T.solver = solver;
    T.omegah = omegah;
    T.omegas = omegas;
    // SteadyGS and ConvexGS visit the elements one after another, with two group barriers per
    // element in a patch group: beyond kMaxGroupGsElements a sweep would take seconds, so large
    // groups refuse them (as the primary solver, and as GDsteady's fallback)
    T.gs_ok = !grouped() || n <= kMaxGroupGsElements;
    if ((solver == 4 || solver == 3) && !T.gs_ok) return -1000;
    // fixed part of the shift: wsfix = -facdt * hs with hs = -dq w (stang_rhs, K = 0)
    double *facdt = P.c(W_FACDT);
    int *edge = P.ci(I_JX);
    const bool cnvx_ss = solver == 3 && is_ssrol;
    const bool trans_prev = d.pvtime == 0 && d.prev && d.tang == 2;
    compute_facdt(P, solver, facdt, (cnvx_ss || trans_prev) ? edge : nullptr);
    // ConvexGS in steady rolling: csv in the columns of the FP32 work arrays W_FLS .. W_FLS + 11
    // (three blocks of 4 mx my doubles; ConvexGS uses none of those arrays), and whether any
    // element takes a leading-edge estimate
    T.csv = nullptr;
    T.edge = edge;
    T.any_edge = false;
    if (cnvx_ss) {
        double *csv = P.c(W_FLS);
        steady_coefs(d, csv);
        T.csv = csv;
        int c = 0;
        FOR_I(i, n) if (edge[i] > 0) c++;
        T.any_edge = block_sumi1(red, c) > 0;
    }
    FOR_I(i, n) {
        iel[i] = igs[i] >= Adhes ? 1 : 0;
        wfx[i] = iel[i] ? -facdt[i] * wx[i] : 0.0;
        wfy[i] = iel[i] ? -facdt[i] * wy[i] : 0.0;
    }
    gsync();
    // K != 0: the tangential displacement of the normal pressure, u(ps_n) - u'(pv_n) (stang_rhs,
    // m_stang.f90:749-951): in steady rolling through the coupling blocks of cs - cv applied to
    // the current pressure; for shifts through cs applied to the pressure minus that of the
    // previous time instance (P = 0, 1), or to the pressure alone (P = 2)
    if (d.ncf >= 6) {
        double *ux = P.c(W_UX), *uy = P.c(W_UY), *un = P.c(W_UN);
        const double *src = pn;
        if (d.tang == 1 && d.pvtime <= 1 && d.prev) {
            const double *pvn = d.prev + 2 * (size_t)n;
            FOR_I(i, n) un[i] = pn[i] - pvn[i];
            src = un;
        }
        prod_tz(*T.op, src, ux, uy, OUT_ALL, igs, d.tang == 3);
        FOR_I(i, n) if (iel[i]) { wfx[i] += ux[i]; wfy[i] += uy[i]; }
        gsync();
    }
    // shifts and transient rolling continuing from the previous time instance (P = 0):
    // wsfix -= u' of the previous tangential tractions, through cs for shifts and through cv
    // (one rolling step) for transient rolling, where elements within one rolling step of
    // their leading edge take the edge estimate of subnd instead (stang_rhs, m_stang.f90:749-951;
    // with identical materials the normal terms vanish, and P = 1 keeps only them)
    if (d.pvtime == 0 && d.prev && (d.tang == 1 || d.tang == 2)) {
        const double *pvx = d.prev, *pvy = d.prev + n;
        const int *igv = (const int *)(d.prev + 3 * (size_t)n);
        double *ux = P.c(W_UX), *uy = P.c(W_UY);
        // cs pv on all elements: u' of the shift, or the edge estimate at ix0 + 1 (facdx = 1)
        prod_t<double>(*T.op, pvx, pvy, ux, uy, OUT_ALL, igs);
        if (d.tang == 1) {
            FOR_I(i, n) if (iel[i]) { wfx[i] -= ux[i]; wfy[i] -= uy[i]; }
        } else {
            double *cvc = P.c(W_FLS);          // 12 columns, overwritten by the solver later
            transient_coefs(d, cvc);
            const size_t bsz = (size_t)4 * mx * my;
            const double *cxx = cvc, *cxy = cvc + bsz, *cyy = cvc + 2 * bsz;
            FOR_I(i, n) {
                if (!iel[i]) continue;
                const int ix0 = edge[i];
                if (ix0 > 0) {
                    if (ix0 + 2 <= mx) {
                        const int je = ix0 + (i / mx) * mx;
                        wfx[i] -= ux[je]; wfy[i] -= uy[je];
                    }
                    continue;
                }
                const int ix = i % mx, iy = i / mx;
                double a0 = 0.0, a1 = 0.0;
                for (int j = 0; j < n; j++) {
                    if (igv[j] < Adhes) continue;
                    const int jx = j % mx, jy = j / mx;
                    const size_t off = (size_t)(ix - jx + mx) + (size_t)(iy - jy + my) * 2 * mx;
                    a0 += cxx[off] * pvx[j] + cxy[off] * pvy[j];
                    a1 += cxy[off] * pvx[j] + cyy[off] * pvy[j];
                }
                wfx[i] -= a0 / d.ga; wfy[i] -= a1 / d.ga;
            }
        }
        gsync();
    }
    // row extents of the contact area for the row sums (solvpt, m_solvpt.f90:51-378, sets them
    // before the solver; the contact area does not change within TANG)
    areas(P);
    int ittang = 0, itgs = 0;
    bool zready = false;
    double *one = P.c(W_ONE);
    while (!zready && ittang < d.maxin) {
        ittang++;
        zready = true;
        int info = 0;
        double errpt = 0.0;
        const int it = solvpt(P, T, info, errpt);
        if (it < 0) return it;
        itgs += it;
        if (info >= 3) { zready = true; ittang = -1; }
        const double tol = sqrt(2.0) * errpt;
        int newins = 0;
        FOR_I(i, n) if (iel[i] && igs[i] == Adhes) {
            double pabs = sqrt(px[i] * px[i] + py[i] * py[i]);
            if (pabs >= d.fstat * pn[i] + tol) {
                newins++;
                igs[i] = Slip;
                px[i] = px[i] * d.fstat * pn[i] / pabs;
                py[i] = py[i] * d.fstat * pn[i] / pabs;
            }
        }
        newins = block_sumi1(red, newins);
        if (newins != 0) zready = false;
        if (zready) {
            areas(P);
            int ii0 = (max(1, mx / 2) - 1) + (max(1, my / 2) - 1) * mx;
            FOR_I(i, n) one[i] = 1.0;
            gsync();
            int blk[2] = {0, 2};
            const double *vv[2] = {nullptr, nullptr};
            int rid[2] = {0, 1};
            double tt[2];
            direct_rowsum(P, ii0, 2, blk, vv, tt, rid, 2);
            const double tol1 = errpt * 2.0 * fabs(tt[0]), tol2 = errpt * 2.0 * fabs(tt[1]);
            int newadh = 0;
            FOR_I(i, n) if (iel[i] && igs[i] == Slip) {
                double ww = sx[i] * px[i] + sy[i] * py[i];
                double tl = tol1 * fabs(px[i]) + tol2 * fabs(py[i]) + errpt * (fabs(sx[i]) + fabs(sy[i]));
                if (ww > tl) { igs[i] = Adhes; newadh++; }
            }
            newadh = block_sumi1(red, newadh);
            if (newadh != 0) zready = false;
            if (info > 0) zready = true;
        }
        gsync();
    }
    if (!zready) ittang = -1;
    itgs_out = itgs;
    if (d.sens >= 3 && !sens_tang(P, T)) return -2000;
    return ittang;
}

// output quantities, soutpt m_soutpt.f90:377-511
template <typename T>
__device__ __noinline__ void soutpt(const PView &P, const Ops<T> &op, double pen, double fntrue, double *out) {
    const PatchDesc &d = *P.d;
    const int mx = P.mx, n = P.n;
    RedSmem &red = P.sm->red;
    int *igs = P.igs();
    double *px = P.c(W_PX), *py = P.c(W_PY), *pn = P.c(W_PN);
    double *ux = P.c(W_UX), *uy = P.c(W_UY), *un = P.c(W_UN), *sx = P.c(W_SX), *sy = P.c(W_SY), *sn = P.c(W_SN);
    const double *h = P.c(W_H);
    FOR_I(i, n) { ux[i] = 0.0; uy[i] = 0.0; un[i] = 0.0; }
    prod_n<T>(op, pn, un, OUT_INT, igs, 3);
    prod_t<T>(op, px, py, ux, uy, OUT_INT, igs);
    // K != 0: the coupling terms of u = A p (all components, m_soutpt.f90:377-511)
    if (d.ncf >= 6) {
        prod_zt(op, px, py, un, true, igs);
        prod_tz(op, pn, ux, uy, OUT_ADDINT, igs, false);
    }
    double a[4] = {0, 0, 0, 0};
    double b[2] = {0, 0};
    double pmax = -1e20;
    int c[3] = {0, 0, 0};
    FOR_I(i, n) {
        const double x = d.xc1 + (i % mx) * d.dx, y = d.yc1 + (i / mx) * d.dy;
        a[0] += pn[i]; a[1] += px[i]; a[2] += py[i];
        a[3] += px[i] * y;
        b[0] += py[i] * x;
        if (igs[i] >= Adhes) b[1] += un[i] * pn[i] + ux[i] * px[i] + uy[i] * py[i];
        pmax = fmax(pmax, pn[i]);
        if (igs[i] == Adhes) c[0]++; else if (igs[i] == Slip) c[1]++; else if (igs[i] == Plast) c[2]++;
        sn[i] = -pen + h[i] + un[i];
        if (igs[i] != Slip) { sx[i] = 0.0; sy[i] = 0.0; }
    }
    block_sum<4>(red, a);
    block_sum<2>(red, b);
    block_sumi<3>(red, c);
    pmax = block_max1(red, pmax);
    const double dxdy = d.dxdy, muscal = d.fstat, tiny = 1e-20;
    const double fn = (d.norm == 0) ? dxdy * a[0] : fntrue;
    // prescribed total forces are reported as prescribed (m_soutpt.f90:427-434)
    const double fxrel = (d.force3 >= 1) ? d.fxrel : dxdy * a[1] / (fn * muscal + tiny);
    const double fyrel = (d.force3 >= 2) ? d.fyrel : dxdy * a[2] / (fn * muscal + tiny);
    double mz = -dxdy * a[3] + dxdy * b[0];
    if (fabs(mz) < 0.5 * d.eps * (muscal * fn + tiny)) mz = 0.0;
    if (glead()) {
        out[O_FN] = fn;
        out[O_FX] = fxrel * (fn * muscal + tiny);
        out[O_FY] = fyrel * (fn * muscal + tiny);
        out[O_MZ] = mz;
        out[O_PEN] = pen;
        out[O_ELEN] = 0.5 * 1e-3 * dxdy * b[1];
        out[O_PMAX] = pmax;
        out[O_NCON] = c[0] + c[1] + c[2];
        out[O_NADH] = c[0];
        out[O_NSLIP] = c[1];
    }
    gsync();
}

// interior elements at the boundary of the potential contact (eldiv_count_atbnd,
// m_gridfunc.f90:437-490, rows and columns)
__device__ __noinline__ int count_atbnd(const PView &P) {
    const int mx = P.mx, my = P.my, n = P.n;
    const int *igs = P.igs();
    int c = 0;
    FOR_I(ii, n) {
        const int ix = ii % mx + 1, iy = ii / mx + 1;
        const bool rowsel = (mx >= 3) ? true : (iy == 1 || iy == my);
        const bool allx = (my >= 3 && (iy == 1 || iy == my));
        const bool colsel = allx || ix == 1 || ix == mx;
        if (rowsel && colsel && igs[ii] >= Adhes) c++;
    }
    return block_sumi1(P.sm->red, c);
}

// ------------------------------------------------------------------------------------------
// the patch solve
// ------------------------------------------------------------------------------------------
// the solve of one patch by this CTA (blk false) or by this CTA and the others of its patch
// group (blk true)
__device__ __noinline__ void solve_patch(const PatchDesc &d, bool blk, unsigned char *smraw, SolverSmem &sm) {
    group_init(blk ? d.nblk : 1, blk ? (int)blockIdx.x : 0, d.gscr);
    const SmemPlan sp = smem_plan(d.fx, d.fy, blk);
    PView P;
    P.d = &d; P.mx = d.mx; P.my = d.my; P.n = d.npot; P.sm = &sm;
    double *out = P.out();
    if (threadIdx.x < kNumPhaseTimers) sm.t[threadIdx.x] = 0;
    if (threadIdx.x == 0) sm.algb = 0.0;
    const long long t_start = clock64();
    unsigned long long g_start;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(g_start));
    Ops<double> op64;
    make_ops<double>(op64, d, smraw, sp);
    op64.cv.tacc = &sm.t[O_T_CONV - O_T_TOTAL];
    op64.cv.bacc = &sm.algb;
    make_twiddles<double>(op64.cv.twx, sp.NX, blk);
    make_twiddles<double>(op64.cv.twy, sp.NY, blk);
    Ops<float> op32;
    const bool mixed = d.precision >= 1;
    if (mixed) {
        make_ops<float>(op32, d, smraw, sp);
        op32.cv.tacc = &sm.t[O_T_CONV - O_T_TOTAL];
        op32.cv.tacc2 = &sm.t[O_T_CONV32 - O_T_TOTAL];
        op32.cv.bacc = &sm.algb;
        make_twiddles<float>(op32.cv.twx, sp.NX, blk);
        make_twiddles<float>(op32.cv.twy, sp.NY, blk);
    }
    gsync();
    int status = ST_OK;
    if (op64.cv.px.nst < 0 || op64.cv.py.nst < 0) {
        if (glead()) { out[O_STATUS] = ST_BADSIZE; out[O_IERR] = -99; }
        return;
    }
    // clear the work columns that the solvers expect at zero
    {
        const int n = d.npot;
        for (int c = W_UX; c < W_NCOL; c++) {
            double *col = P.c(c);
            FOR_I(i, n) col[i] = 0.0;
        }
        FOR_I(i, n) { P.ci(I_OLD)[i] = 0; P.ci(I_IEL)[i] = 0; }
    }
    gsync();
    setup_patch(P);
    double pen = d.pen, fntrue = d.fntrue;
    // sensitivities [out * 4 + in] (out Fn, Fx, Fy, Mz; in pen, cksi, ceta, cphi): those of the
    // previous solve on a warm start, with the reference's resets (m_sdis.f90:754-766)
    double sens[16];
    for (int k = 0; k < 16; k++) sens[k] = d.sens0[k];
    if (d.iestim == 0) for (int io = 1; io < 4; io++) sens[io * 4] = 0.0;
    if (d.iestim == 0 && (d.norm != 1 || d.ihertz != 0)) sens[0] = 0.0;
    if (d.iestim == 0 || d.iestim == 2)
        for (int io = 0; io < 4; io++) for (int ji = 1; ji < 4; ji++) sens[io * 4 + ji] = 0.0;
    int itnorm = 0, ittang = 0, itcg = 0, itgs = 0, solver = 0, nconv32 = 0, nconv64 = 0, nls = 0;
    // creepages and Newton-Raphson sensitivities: a fresh start takes cksi = 1e-6 (and ceta = 0
    // for F = 2) and zero sensitivities when total forces are prescribed (m_sdis.f90:754-766)
    TangRun T;
    T.op = &op64; T.o32 = mixed ? &op32 : nullptr; T.eps = d.eps; T.eps32 = d.eps32;
    T.nconv = 0; T.nconv32 = 0; T.nls = 0;
    T.solver = 0; T.fntrue = fntrue;
    T.cksi = d.cksi; T.ceta = d.ceta;
    T.sens = sens;
    T.maxgs = d.maxgs; T.p0x = nullptr; T.p0y = nullptr;
    if (d.iestim == 0 || d.iestim == 2) {
        if (d.force3 >= 1) T.cksi = 1e-6;
        if (d.force3 == 2) T.ceta = 0.0;
    }
    // the Panagiotopoulos process (panprc, m_scontc.f90:356-553): NORM and TANG alternately until
    // the tractions change by less than 5 eps (rms) between two passes, at most maxout passes; one
    // pass for identical materials (K = 0, maxout = 1)
    const int n = d.npot;
    int *igs = P.igs();
    double *px = P.c(W_PX), *py = P.c(W_PY), *pn = P.c(W_PN);
    double *o1x = P.c(W_O1X), *o1y = P.c(W_O1Y), *o1n = P.c(W_O1N);
    const bool outer = d.maxout > 1;
    if (outer) {
        FOR_I(i, n) { o1x[i] = px[i]; o1y[i] = py[i]; o1n[i] = pn[i]; }
        gsync();
    }
    int itout = 0;
    double difid = 1.0, dif = 200.0 * difid;
    while (dif > difid && itout < d.maxout && itnorm >= 0 && ittang >= 0) {
        itout++;
        // NORM (skipped for Hertzian traction bounds B = 2, 3)
        const long long t_norm0 = clock64();
        if (!(d.bound >= 2 && d.bound <= 4 && d.ihertz >= 1)) {
            // the normal problem is a small part of a solve: FP64 in both forms, so that the mixed
            // form starts its tangential iteration from exactly the same pressures.  K != 0: the
            // normal displacement of the current tangential tractions joins the undeformed
            // distance
            const double *htang = nullptr;
            if (d.ncf >= 6) {
                double *un = P.c(W_UN);
                prod_zt(op64, px, py, un, false, igs);
                htang = un;
            }
            int it = 0, itc = 0;
            it = snorm<double>(P, op64, d.maxgs, d.maxin, d.eps, pen, itc, nconv64, htang);
            itcg = itc;
            if (it == -2) status |= ST_NORMCG_DIV;
            if (it >= 0) itnorm += it; else itnorm = -1;
            if (d.norm == 0) {
                double s = 0; FOR_I(i, n) s += pn[i];
                fntrue = d.dxdy * block_sum1(sm.red, s);
                T.fntrue = fntrue;
            }
            // d Fn / d pen (S >= 2, m_snorm.f90:357-368); the reference re-evaluates the normal
            // displacements of the final pressures on small grids (npot < 700)
            if (it != -2 && d.sens >= 2) {
                if (d.npot < 700) prod_n<double>(op64, pn, P.c(W_DD), OUT_ALL, igs, 3);
                if (!sens_norm(P, op64, pen, fntrue, nconv64, sens[0])) { status |= ST_NORMCG_DIV; itnorm = -1; }
            } else if (it != -2) {
                sens[0] = 0.0;
            }
        }
        if (threadIdx.x == 0) sm.t[O_T_NORM - O_T_TOTAL] += clock64() - t_norm0;
        if (status != ST_OK) break;
        // clear the exterior tractions, count the contact area (TANG follows NORM also when NORM
        // reached maxin, as in the reference; the loop then ends)
        int ncon = 0;
        FOR_I(i, n) {
            if (igs[i] <= Exter) { pn[i] = 0.0; px[i] = 0.0; py[i] = 0.0; }
            else ncon++;
        }
        ncon = block_sumi1(sm.red, ncon);
        if (d.tang == 0 || ncon <= 0) {
            dif = 0.0;
        } else {
            const long long t_tang0 = clock64();
            int itg = 0;
            const int it = stang(P, T, itg);
            solver = T.solver;
            itgs = itg;
            if (it == -1000) status |= ST_UNSUPPORTED;
            if (it == -2000) status |= ST_NOBRACKET;
            if (it >= 0) ittang += it; else ittang = -1;
            if (threadIdx.x == 0) sm.t[O_T_TANG - O_T_TOTAL] += clock64() - t_tang0;
            if (status != ST_OK) break;
            if (outer) {
                // change of the tractions over the contact area, all components (gf3_rms AllInt)
                double a[2] = {0.0, 0.0};
                int c = 0;
                FOR_I(i, n) {
                    if (igs[i] < Adhes) continue;
                    const double ex = px[i] - o1x[i], ey = py[i] - o1y[i], en = pn[i] - o1n[i];
                    a[0] += ex * ex + ey * ey + en * en;
                    a[1] += px[i] * px[i] + py[i] * py[i] + pn[i] * pn[i];
                    c += 3;
                }
                block_sum<2>(sm.red, a);
                c = block_sumi1(sm.red, c);
                dif = sqrt(a[0] / max(1, c));
                difid = 5.0 * d.eps * sqrt(a[1] / max(1, c));
                FOR_I(i, n) { o1x[i] = px[i]; o1y[i] = py[i]; o1n[i] = pn[i]; }
                gsync();
            }
        }
        if (status != ST_OK) break;
    }
    nconv64 += T.nconv; nconv32 += T.nconv32; nls += T.nls;
    soutpt<double>(P, op64, pen, fntrue, out);
    int atb = count_atbnd(P);
    // the solution, kept in device memory for the problem's next warm start or time instance
    if (d.save) {
        const int n = d.npot;
        const int *igs = P.igs();
        const double *px = P.c(W_PX), *py = P.c(W_PY), *pn = P.c(W_PN);
        int *sg = (int *)(d.save + 3 * (size_t)n);
        FOR_I(i, n) { d.save[i] = px[i]; d.save[n + i] = py[i]; d.save[2 * (size_t)n + i] = pn[i]; sg[i] = igs[i]; }
        gsync();
    }
    // a barrier of the group that gave up (error flag in the group scratch)
    if (blk && ((volatile unsigned *)g_grp.bar)[2] != 0u) status |= ST_GROUPFAIL;
    if (glead()) {
        int ierr;
        if (status != ST_OK) ierr = -99;
        else if (itnorm < 0) ierr = -27;
        else if (ittang < 0) ierr = -28;
        else ierr = atb;
        out[O_IERR] = ierr;
        out[O_ITNORM] = itnorm;
        out[O_ITTANG] = ittang;
        out[O_ITCG] = itcg;
        out[O_ITGS] = itgs;
        out[O_SOLVER] = solver;
        out[O_NCONV32] = nconv32;
        out[O_NCONV64] = nconv64;
        out[O_NLS] = nls;
        out[O_STATUS] = status;
        sm.t[0] = clock64() - t_start;
        for (int k = 0; k < kNumPhaseTimers; k++) out[O_T_TOTAL + k] = (double)sm.t[k];
        out[O_ALGB] = sm.algb;
        unsigned long long g_end;
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(g_end));
        out[O_TSTART] = (double)g_start;
        out[O_TEND] = (double)g_end;
        out[O_CKSI] = T.cksi;
        out[O_CETA] = T.ceta;
        for (int k = 0; k < 16; k++) out[O_SENS + k] = sens[k];
    }
    // completion signal for the host: after the group barrier every result of the patch is in
    // its io block; the system-scope fence orders them before the flag
    if (d.done) {
        gsync();
        if (glead()) {
            __threadfence_system();
            *(volatile int *)d.done = 1;
        }
    }
}

// grid: one CTA per listed patch (mode 0); the nblk CTAs of one patch group (mode 1, cooperative
// launch, list[0] is the patch); or a persistent grid (mode 2) whose CTAs take the nlist listed
// patches in list order from the queue counter *queue until none is left, so that the SMs that
// finish early take the next patch instead of idling
__global__ void __launch_bounds__(kThreads, 2) k_solve(const PatchDesc *descs, const int *list, int mode, int nlist,
                                                       int *queue) {
    extern __shared__ __align__(16) unsigned char smraw[];
    __shared__ SolverSmem sm;
    __shared__ int next;
    if (mode == 2) {
        for (;;) {
            if (threadIdx.x == 0) next = atomicAdd(queue, 1);
            __syncthreads();
            const int k = next;
            __syncthreads();
            if (k >= nlist) break;
            solve_patch(descs[list[k]], false, smraw, sm);
            __syncthreads();
        }
        return;
    }
    solve_patch(descs[list[mode ? 0 : blockIdx.x]], mode != 0, smraw, sm);
}

// ------------------------------------------------------------------------------------------
// host side
// ------------------------------------------------------------------------------------------
static size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

int opt_fft_size(int fft_size) {
    static const int kpat[9][8] = {
        {-2, 1, 0, 0, 0, 4, 3, 3},   {-5, 3, 0, 0, 0, 32, 27, 3},  {-1, -1, 1, 0, 0, 6, 5, 5},
        {-4, 1, 1, 0, 0, 16, 15, 5}, {0, -3, 2, 0, 0, 27, 25, 5},  {-3, 0, 0, 1, 0, 8, 7, 7},
        {1, -1, -1, 1, 0, 15, 14, 7}, {-1, 2, -1, 0, 0, 10, 9, 5}, {-2, -1, 0, 0, 1, 12, 11, 11}};
    int k2 = 0;
    while ((1L << k2) < fft_size) k2++;
    long prod = 1L << k2;
    int kf[5] = {k2, 0, 0, 0, 0};
    bool changed = true;
    while (changed) {
        changed = false;
        for (int ip = 0; ip < 9; ip++) {
            const int *kp = kpat[ip];
            if (kp[7] > 7) continue;
            for (;;) {
                bool ok = true;
                for (int f = 0; f < 5; f++) if (kf[f] + kp[f] < 0) ok = false;
                if (!(ok && (long)kp[6] * prod >= (long)kp[5] * fft_size)) break;
                for (int f = 0; f < 5; f++) kf[f] += kp[f];
                prod = (long)kp[6] * prod / kp[5];
                changed = true;
            }
        }
    }
    return (int)prod;
}

PatchSizes patch_sizes(int mx, int my, int fx, int fy, int nblk, int ncf) {
    PatchSizes s;
    const size_t n = (size_t)mx * my;
    const size_t ksz = (size_t)(fx + 1) * (fy + 1);
    s.io = align256(io_doubles((int)n) * sizeof(double));
    s.cf = align256((size_t)ncf * 4 * n * sizeof(double));
    s.spec64 = align256((size_t)spectra_count(ncf) * ksz * sizeof(double));
    s.spec32 = align256((size_t)spectra_count(ncf) * ksz * sizeof(float));
    size_t wkn = (size_t)(W_NCOL - kIoCols) * n;
    const size_t specscratch = spectra_scratch_doubles(mx, my, fx, fy) + 4 * n;   // k_spectra
    if (wkn < specscratch) wkn = specscratch;
    s.wk = align256(wkn * sizeof(double));
    s.wki = align256((size_t)(I_NCOL - 1) * n * sizeof(int));
    s.rbuf = align256((size_t)2 * (fx + 1) * my * 16);
    s.gscr = nblk > 1 ? group_tw(nblk, mx, my, fx, fy).total : 0;
    s.work = s.cf + s.spec64 + s.spec32 + s.wk + s.wki + s.rbuf + s.gscr;
    return s;
}

void carve_patch(PatchDesc &d, char *io, char *work) {
    const PatchSizes s = patch_sizes(d.mx, d.my, d.fx, d.fy, d.nblk, d.ncf);
    d.io = (double *)io;
    char *p = work;
    d.cf = (const double *)p; p += s.cf;
    d.spec64 = (const double *)p; p += s.spec64;
    d.spec32 = (const float *)p; p += s.spec32;
    d.wk = (double *)p; p += s.wk;
    d.wki = (int *)p; p += s.wki;
    d.rbuf = (void *)p; p += s.rbuf;
    d.gscr = s.gscr ? (void *)p : nullptr; p += s.gscr;
}

size_t solve_smem_bytes(int fx, int fy, bool group) { return smem_plan(fx, fy, group).total; }

static std::mutex g_attr_mu;
static size_t g_attr_solve = 0, g_attr_spec = 0;

static cudaError_t ensure_smem_attr(size_t need) {
    std::lock_guard<std::mutex> lk(g_attr_mu);
    cudaError_t e = cudaSuccess;
    if (need > g_attr_solve) {
        e = cudaFuncSetAttribute(k_solve, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)need);
        if (e != cudaSuccess) return e;
        g_attr_solve = need;
    }
    if (need > g_attr_spec) {
        e = cudaFuncSetAttribute(k_spectra, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)need);
        if (e != cudaSuccess) return e;
        g_attr_spec = need;
    }
    return e;
}

// dynamic shared memory a CTA of the patch kernels may use on the current device: the
// opt-in maximum per block less the kernels' static shared memory
size_t max_dynamic_smem() {
    static std::mutex mu;
    static size_t cached = 0;
    std::lock_guard<std::mutex> lk(mu);
    if (cached) return cached;
    int dev = 0, optin = 0;
    cudaFuncAttributes fa, fb;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess ||
        cudaFuncGetAttributes(&fa, k_solve) != cudaSuccess || cudaFuncGetAttributes(&fb, k_spectra) != cudaSuccess) {
        cudaGetLastError();
        return 227 * 1024 - 16384;     // no device: a conservative bound
    }
    cached = (size_t)optin - std::max(fa.sharedSizeBytes, fb.sharedSizeBytes);
    return cached;
}

// grids above this many elements are solved by a patch group when the choice is automatic:
// one CTA would spend seconds per solve where a group spreads the work over many SMs
constexpr int kMaxSingleCtaElements = 44100;     // 210 x 210

int group_size(int mx, int my, int fx, int fy, int requested) {
    const size_t lim = max_dynamic_smem();
    const bool fits1 = smem_plan(fx, fy, false).total <= lim;
    if (requested == 1) return fits1 ? 1 : -1;
    if (requested <= 0 && fits1 && mx * my <= kMaxSingleCtaElements) return 1;
    const size_t sm = smem_plan(fx, fy, true).total;
    if (sm > lim) return -1;
    if (ensure_smem_attr(sm) != cudaSuccess) { cudaGetLastError(); return -1; }
    int dev = 0, nsm = 0, occ_a = 0, occ_b = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_a, k_solve, kThreads, sm) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_b, k_spectra, kThreads, sm) != cudaSuccess) {
        cudaGetLastError();
        return -1;
    }
    const int cap = nsm * std::min(occ_a, occ_b);
    if (cap < 2) return -1;
    int want = requested >= 2 ? requested : (mx * my + kThreads - 1) / kThreads;
    return std::max(2, std::min(want, cap));
}

int engine_plan(const PatchDesc *hdesc, int n, const unsigned char *compute_ic, EnginePlan &pl) {
    pl = EnginePlan();
    if (n <= 0) return 0;
    auto smem_of = [&](int i) { return solve_smem_bytes(hdesc[i].fx, hdesc[i].fy, hdesc[i].nblk > 1); };
    // order: influence list first, then the single-CTA patches, largest first (the queue of the
    // persistent solve), then the patch groups
    std::vector<int> ic_list, ic_single, order, groups;
    for (int i = 0; i < n; i++) {
        if (compute_ic[i]) { ic_list.push_back(i); if (hdesc[i].nblk <= 1) ic_single.push_back(i); }
        if (hdesc[i].nblk > 1) groups.push_back(i); else order.push_back(i);
    }
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return hdesc[a].npot > hdesc[b].npot; });
    pl.nsingle = (int)order.size();
    order.insert(order.end(), groups.begin(), groups.end());
    pl.all = ic_list;
    pl.all.insert(pl.all.end(), ic_single.begin(), ic_single.end());
    pl.all.insert(pl.all.end(), order.begin(), order.end());
    pl.n_ic = (int)ic_list.size();
    pl.n_ics = (int)ic_single.size();
    for (int i = 0; i < n; i++) pl.maxsm = std::max(pl.maxsm, smem_of(i));
    cudaError_t e = ensure_smem_attr(pl.maxsm);
    if (e != cudaSuccess) return (int)e;
    if (!ic_list.empty()) {
        int maxn = 0;
        for (int i : ic_list) maxn = std::max(maxn, 4 * hdesc[i].mx * hdesc[i].my);
        pl.ginf = dim3(std::min(64, (maxn + kThreads - 1) / kThreads), (unsigned)ic_list.size());
        for (int i : ic_single) pl.sm_spec = std::max(pl.sm_spec, smem_of(i));
    }
    if (pl.nsingle > 0) {
        for (int k = 0; k < pl.nsingle; k++) pl.sm_solve = std::max(pl.sm_solve, smem_of(order[k]));
        int dev = 0, nsm = 0, occ = 0;
        if ((e = cudaGetDevice(&dev)) != cudaSuccess) return (int)e;
        if ((e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return (int)e;
        if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_solve, kThreads, pl.sm_solve)) != cudaSuccess)
            return (int)e;
        pl.grid_solve = std::max(1, std::min(pl.nsingle, nsm * std::max(1, occ)));
    }
    for (int k = pl.nsingle; k < (int)order.size(); k++) {
        const int i = order[k];
        EnginePlan::Group g;
        g.k = k; g.nblk = hdesc[i].nblk; g.sm = smem_of(i); g.gscr = hdesc[i].gscr; g.ic = compute_ic[i] != 0;
        pl.groups.push_back(g);
    }
    pl.kernels = (pl.n_ic > 0) + (pl.n_ics > 0) + (pl.nsingle > 0);
    for (const auto &g : pl.groups) pl.kernels += 1 + (g.ic ? 1 : 0);
    return 0;
}

int engine_launch(const EnginePlan &pl, PatchDesc *ddesc, int *d_list, cudaStream_t stream, EngineTimer *timer) {
    if (timer) timer->nlaunch = 0;
    if (pl.all.empty()) return 0;
    auto mark = [&](int kind, bool after) {
        if (!timer || timer->nlaunch >= EngineTimer::kMax) return;
        cudaEventRecord(timer->ev[2 * timer->nlaunch + (after ? 1 : 0)], stream);
        if (after) { timer->kind[timer->nlaunch] = kind; timer->nlaunch++; }
    };
    cudaError_t e;
    const int *d_ic = d_list;
    const int *d_ics = d_list + pl.n_ic;
    const int *d_order = d_ics + pl.n_ics;
    if (pl.n_ic > 0) {
        mark(0, false);
        k_influence<<<pl.ginf, kThreads, 0, stream>>>(ddesc, d_ic);
        mark(0, true);
        if (pl.n_ics > 0) {
            mark(1, false);
            k_spectra<<<(unsigned)pl.n_ics, kThreads, pl.sm_spec, stream>>>(ddesc, d_ics, 0);
            mark(1, true);
        }
    }
    // the single-CTA patches: one persistent launch of (co-resident CTAs of the device) CTAs that
    // take the patches from a queue in device memory, largest first; the queue counter follows
    // the lists in d_list
    mark(2, false);
    if (pl.nsingle > 0) {
        int *queue = d_list + pl.all.size();
        if ((e = cudaMemsetAsync(queue, 0, sizeof(int), stream)) != cudaSuccess) return (int)e;
        k_solve<<<pl.grid_solve, kThreads, pl.sm_solve, stream>>>(ddesc, d_order, 2, pl.nsingle, queue);
    }
    // patch groups: cooperative launches, one patch at a time on the caller's stream after
    // all single-CTA work, so that nothing else of this library shares the SMs with them
    for (const auto &g : pl.groups) {
        if ((e = cudaMemsetAsync(g.gscr, 0, 256, stream)) != cudaSuccess) return (int)e;
        const int *lp = d_order + g.k;
        int grp = 1, nl = 1;
        int *noq = nullptr;
        void *args[5] = {(void *)&ddesc, (void *)&lp, (void *)&grp, (void *)&nl, (void *)&noq};
        if (g.ic) {
            e = cudaLaunchCooperativeKernel((const void *)k_spectra, dim3(g.nblk), dim3(kThreads), args, g.sm, stream);
            if (e != cudaSuccess) return (int)e;
            if ((e = cudaMemsetAsync(g.gscr, 0, 256, stream)) != cudaSuccess) return (int)e;
        }
        e = cudaLaunchCooperativeKernel((const void *)k_solve, dim3(g.nblk), dim3(kThreads), args, g.sm, stream);
        if (e != cudaSuccess) return (int)e;
    }
    mark(2, true);
    return (int)cudaGetLastError();
}

void count_launches(long long k) { g_launches += k; }

int engine_run(const PatchDesc *hdesc, PatchDesc *ddesc, int n, const unsigned char *compute_ic,
               int *d_list, cudaStream_t stream, EngineTimer *timer) {
    if (timer) timer->nlaunch = 0;
    if (n <= 0) return 0;
    EnginePlan pl;
    int rc = engine_plan(hdesc, n, compute_ic, pl);
    if (rc != 0) return rc;
    cudaError_t e = cudaMemcpyAsync(d_list, pl.all.data(), pl.all.size() * sizeof(int), cudaMemcpyHostToDevice, stream);
    if (e != cudaSuccess) return (int)e;
    // the host vector must outlive the asynchronous copy
    e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) return (int)e;
    rc = engine_launch(pl, ddesc, d_list, stream, timer);
    if (rc == 0) g_launches += pl.kernels;
    return rc;
}

} // namespace cgb
