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
__device__ inline void corner(int ix, int iy, double dx, double dy, double &x, double &y, double &r) {
    x = (double)(float)ix * dx - 0.5 * dx;
    y = (double)(float)iy * dy - 0.5 * dy;
    r = sqrt(x * x + y * y);
}

// grid: (blocks per patch, number of listed patches); list[] gives the patch indices
__global__ void __launch_bounds__(kThreads) k_influence(const PatchDesc *descs, const int *list) {
    const PatchDesc &d = descs[list[blockIdx.y]];
    const int mx = d.mx, my = d.my;
    const int total = 4 * mx * my;
    const double pi = 3.14159265358979323846;
    const double e1 = (1.0 - d.nu) / pi, e2 = 1.0 / pi, e3 = d.nu / pi;
    const double dx = d.dx, dy = d.dy, tolx = dx * 1e-10;
    const int iy0 = (my == 1) ? 0 : -my;
    double *cf = const_cast<double *>(d.cf);
    const size_t bsz = (size_t)total;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
        const int ix = t % (2 * mx) - mx, iy = t / (2 * mx) - my;
        double c11 = 0, c12 = 0, c22 = 0, c33 = 0;
        if (iy >= iy0) {
            double x00, y00, r00, x01, y01, r01, x10, y10, r10, x11, y11, r11;
            corner(ix, iy, dx, dy, x00, y00, r00);
            corner(ix, iy + 1, dx, dy, x01, y01, r01);
            corner(ix + 1, iy, dx, dy, x10, y10, r10);
            corner(ix + 1, iy + 1, dx, dy, x11, y11, r11);
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
        }
        cf[0 * bsz + t] = c11;
        cf[1 * bsz + t] = c12;
        cf[2 * bsz + t] = c22;
        cf[3 * bsz + t] = c33;
    }
}

// ------------------------------------------------------------------------------------------
// shared-memory plan of a patch block
// ------------------------------------------------------------------------------------------
struct SmemPlan {
    int NX, NY, nmax;
    size_t off_tw64x, off_tw64y, off_tw32x, off_tw32y, off_wbuf, total;
};

// single CTA (blk false): twiddle tables and one buffer region of 4 * max(NX, NY) complex
// per warp in shared memory.  Patch group (blk true): one buffer region per CTA, the twiddle
// tables live in the group scratch in global memory.
__host__ __device__ inline SmemPlan smem_plan(int fx, int fy, bool blk = false) {
    SmemPlan s;
    s.NX = 2 * fx; s.NY = 2 * fy; s.nmax = s.NX > s.NY ? s.NX : s.NY;
    size_t o = 0;
    if (blk) {
        s.off_tw64x = s.off_tw64y = s.off_tw32x = s.off_tw32y = 0;
        s.off_wbuf = 0;
        s.total = (size_t)4 * s.nmax * 16;
        return s;
    }
    s.off_tw64x = o; o += (size_t)s.NX * 16;
    s.off_tw64y = o; o += (size_t)s.NY * 16;
    s.off_tw32x = o; o += (size_t)s.NX * 8;
    s.off_tw32y = o; o += (size_t)s.NY * 8;
    o = (o + 15) & ~(size_t)15;
    s.off_wbuf = o; o += (size_t)kWarps * 4 * s.nmax * 16;
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
    for (int b = 0; b < 7; b++) op.K[b] = base + b * ksz;
}

// ------------------------------------------------------------------------------------------
// spectra of the coefficient blocks and of the FFT preconditioners (one block per patch)
// ------------------------------------------------------------------------------------------
// real, quadrant-symmetric conv-size spectrum of a spatial block src (layout of cf:
// (dx + mx) + (dy + my) * 2mx); offsets |dx| <= mx-1, |dy| <= my-1 are placed at
// (dx mod NX, dy mod NY).  S: scratch of nkx * NY complex.
__device__ __noinline__ void block_spectrum(const Conv<double> &cv, const double *src, double2 *S, double *K64,
                                            float *K32, double2 *a, double2 *b) {
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
            K64[o] = z[ky].x;
            K32[o] = (float)z[ky].x;
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

// leading-edge fraction facdt (sxbnd, m_leadedge.f90:92-332) for rolling direction chi = 0
__device__ __noinline__ void compute_facdt(const PView &P, int solver, double *facdt) {
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
            if (!is_roll) facdt[ii] = 1.0;
            else if (igs[ii] <= Exter) facdt[ii] = 0.0;
            else if (ix + 2 > mx) facdt[ii] = 1.0;
            else {
                const double xbnd = d.xc1 + (ixb - 1) * d.dx + fxdfac * d.dx;
                const double x = d.xc1 + (ix - 1) * d.dx;
                facdt[ii] = fmin(1.0, (xbnd - x) / d.dq);
            }
        }
    }
    gsync();
}

constexpr int kMaxGroupGsElements = 40000;

// TANG, m_stang.f90:28-746 for Coulomb friction and prescribed creepages.
// Returns ittang; -1000 when the reference would pick ConvexGS, -2000 on a failed line search.
// With o32 (mixed precision): GDsteady runs once with FP32 direction products and FP64
// residual replacement; TangCG runs an FP32 pass to eps32 followed by an FP64 pass.
__device__ __noinline__ int stang(const PView &P, const Ops<double> &op, const Ops<float> *o32, double eps,
                                  double eps32, int &itgs_out, int &solver_out, int &nconv, int &nconv32, int &nls) {
    const PatchDesc &d = *P.d;
    const int mx = P.mx, my = P.my, n = P.n;
    RedSmem &red = P.sm->red;
    int *igs = P.igs(), *iel = P.ci(I_IEL);
    const bool is_ssrol = d.tang == 3;
    double *px = P.c(W_PX), *py = P.c(W_PY), *pn = P.c(W_PN), *sx = P.c(W_SX), *sy = P.c(W_SY);
    double *wsx = P.c(W_WSX), *wsy = P.c(W_WSY), *wx = P.c(W_WX), *wy = P.c(W_WY);
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
    solver_out = solver;
    if (solver == 3) return -1000;
    // SteadyGS visits the elements one after another, with two group barriers per element in a
    // patch group: beyond kMaxGroupGsElements a sweep would take seconds, so large groups
    // refuse it (as the primary solver, and as GDsteady's fallback below)
    const bool gs_ok = !grouped() || n <= kMaxGroupGsElements;
    if (solver == 4 && !gs_ok) return -1000;
    // fixed part of the shift: wsfix = -facdt * hs with hs = -dq w (stang_rhs, K = 0)
    double *facdt = P.c(W_DSCL);
    compute_facdt(P, solver, facdt);
    FOR_I(i, n) {
        iel[i] = igs[i] >= Adhes ? 1 : 0;
        wsx[i] = iel[i] ? -facdt[i] * wx[i] : 0.0;
        wsy[i] = iel[i] ? -facdt[i] * wy[i] : 0.0;
    }
    gsync();
    int ittang = 0, itgs = 0;
    bool zready = false;
    double *one = P.c(W_ONE);
    while (!zready && ittang < d.maxin) {
        ittang++;
        zready = true;
        int info = 0, it = 0;
        double errpt = 0.0;
        if (solver == 4) {
            it = stdygs(P, eps, d.maxgs, omegah, omegas, info, errpt);
        } else if (solver == 7) {
            bool lstagn = false;
            it = gdsteady<double>(P, op, d.maxgs, eps, errpt, lstagn, nconv, nls, o32, nconv32);
            if (it == -100000) return -2000;
            if (lstagn && !gs_ok) return -1000;
            if (lstagn) it = stdygs(P, eps, d.maxgs, omegah, omegas, info, errpt);
        } else {
            if (o32) {
                it = tangcg<float>(P, *o32, o32->K[5], o32->K[6], d.maxgs, eps32, errpt, nconv32);
                itgs += it > 0 ? it : 0;
            }
            it = tangcg<double>(P, op, op.K[5], op.K[6], d.maxgs, eps, errpt, nconv);
        }
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
    const double fxrel = dxdy * a[1] / (fn * muscal + tiny);
    const double fyrel = dxdy * a[2] / (fn * muscal + tiny);
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
// grid: one CTA per listed patch (group == 0), or the nblk CTAs of one patch group (group
// != 0, cooperative launch, list[0] is the patch)
__global__ void __launch_bounds__(kThreads, 2) k_solve(const PatchDesc *descs, const int *list, int group) {
    extern __shared__ __align__(16) unsigned char smraw[];
    __shared__ SolverSmem sm;
    const PatchDesc &d = descs[list[group ? 0 : blockIdx.x]];
    const bool blk = group != 0;
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
    int itnorm = 0, ittang = 0, itcg = 0, itgs = 0, solver = 0, nconv32 = 0, nconv64 = 0, nls = 0;
    // NORM (skipped for Hertzian traction bounds B = 2, 3)
    long long t_norm0 = clock64();
    if (!(d.bound >= 2 && d.bound <= 4 && d.ihertz >= 1)) {
        // the normal problem is a small part of a solve: FP64 in both forms, so that the mixed
        // form starts its tangential iteration from exactly the same pressures
        int it = 0, itc = 0;
        it = snorm<double>(P, op64, d.maxgs, d.maxin, d.eps, pen, itc, nconv64);
        itcg += itc;
        if (it == -2) status |= ST_NORMCG_DIV;
        itnorm = it >= 0 ? it : -1;
        if (d.norm == 0) {
            double s = 0; FOR_I(i, d.npot) s += P.c(W_PN)[i];
            fntrue = d.dxdy * block_sum1(sm.red, s);
        }
    }
    if (threadIdx.x == 0) sm.t[O_T_NORM - O_T_TOTAL] = clock64() - t_norm0;
    // clear the exterior tractions, count the contact area
    int ncon = 0;
    {
        int *igs = P.igs();
        double *px = P.c(W_PX), *py = P.c(W_PY), *pn = P.c(W_PN);
        FOR_I(i, d.npot) {
            if (igs[i] <= Exter) { pn[i] = 0.0; px[i] = 0.0; py[i] = 0.0; }
            else ncon++;
        }
        ncon = block_sumi1(sm.red, ncon);
    }
    long long t_tang0 = clock64();
    if (d.tang != 0 && ncon > 0 && itnorm >= 0) {
        int it = 0, itg = 0;
        it = stang(P, op64, mixed ? &op32 : nullptr, d.eps, d.eps32, itg, solver, nconv64, nconv32, nls);
        itgs += itg;
        if (it == -1000) status |= ST_UNSUPPORTED;
        if (it == -2000) status |= ST_NOBRACKET;
        ittang = it >= 0 ? it : -1;
    }
    if (threadIdx.x == 0) sm.t[O_T_TANG - O_T_TOTAL] = clock64() - t_tang0;
    soutpt<double>(P, op64, pen, fntrue, out);
    int atb = count_atbnd(P);
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
    }
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

PatchSizes patch_sizes(int mx, int my, int fx, int fy, int nblk) {
    PatchSizes s;
    const size_t n = (size_t)mx * my;
    const size_t ksz = (size_t)(fx + 1) * (fy + 1);
    s.io = align256(io_doubles((int)n) * sizeof(double));
    s.cf = align256(16 * n * sizeof(double));
    s.spec64 = align256(7 * ksz * sizeof(double));
    s.spec32 = align256(7 * ksz * sizeof(float));
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
    const PatchSizes s = patch_sizes(d.mx, d.my, d.fx, d.fy, d.nblk);
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

int group_size(int mx, int my, int fx, int fy, int requested) {
    const size_t lim = max_dynamic_smem();
    const bool fits1 = smem_plan(fx, fy, false).total <= lim;
    if (requested == 1) return fits1 ? 1 : -1;
    if (requested <= 0 && fits1) return 1;
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

// side streams of the calling host thread (created once, never destroyed before exit)
struct SideStreams {
    static constexpr int kN = 16;
    cudaStream_t s[kN];
    cudaEvent_t fork, join[kN];
    bool ok = false;
};

static SideStreams &side_streams() {
    thread_local SideStreams ss;
    thread_local bool init = false;
    if (!init) {
        init = true;
        bool ok = cudaEventCreateWithFlags(&ss.fork, cudaEventDisableTiming) == cudaSuccess;
        for (int k = 0; k < SideStreams::kN && ok; k++) {
            ok = cudaStreamCreateWithFlags(&ss.s[k], cudaStreamNonBlocking) == cudaSuccess &&
                 cudaEventCreateWithFlags(&ss.join[k], cudaEventDisableTiming) == cudaSuccess;
        }
        ss.ok = ok;
    }
    return ss;
}

int engine_run(const PatchDesc *hdesc, PatchDesc *ddesc, int n, const unsigned char *compute_ic,
               int *d_list, cudaStream_t stream, EngineTimer *timer) {
    if (timer) timer->nlaunch = 0;
    if (n <= 0) return 0;
    auto mark = [&](int kind, bool after) {
        if (!timer || timer->nlaunch >= EngineTimer::kMax) return;
        cudaEventRecord(timer->ev[2 * timer->nlaunch + (after ? 1 : 0)], stream);
        if (after) { timer->kind[timer->nlaunch] = kind; timer->nlaunch++; }
    };
    auto smem_of = [&](int i) { return solve_smem_bytes(hdesc[i].fx, hdesc[i].fy, hdesc[i].nblk > 1); };
    // order: influence list first, then the single-CTA patches grouped by shared-memory class,
    // largest first, then the patch groups
    std::vector<int> ic_list, ic_single, order, groups;
    for (int i = 0; i < n; i++) {
        if (compute_ic[i]) { ic_list.push_back(i); if (hdesc[i].nblk <= 1) ic_single.push_back(i); }
        if (hdesc[i].nblk > 1) groups.push_back(i); else order.push_back(i);
    }
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        size_t sa = smem_of(a), sb = smem_of(b);
        if (sa != sb) return sa > sb;
        return hdesc[a].npot > hdesc[b].npot;
    });
    const int nsingle = (int)order.size();
    order.insert(order.end(), groups.begin(), groups.end());
    std::vector<int> all(ic_list);
    all.insert(all.end(), ic_single.begin(), ic_single.end());
    all.insert(all.end(), order.begin(), order.end());
    cudaError_t e = cudaMemcpyAsync(d_list, all.data(), all.size() * sizeof(int), cudaMemcpyHostToDevice, stream);
    if (e != cudaSuccess) return (int)e;
    // the host vector must outlive the asynchronous copy
    e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) return (int)e;
    const int *d_ic = d_list;
    const int *d_ics = d_list + ic_list.size();
    const int *d_order = d_ics + ic_single.size();
    size_t maxsm = 0;
    for (int i = 0; i < n; i++) maxsm = std::max(maxsm, smem_of(i));
    e = ensure_smem_attr(maxsm);
    if (e != cudaSuccess) return (int)e;
    if (!ic_list.empty()) {
        int maxn = 0;
        size_t smax = 0;
        for (int i : ic_list) maxn = std::max(maxn, 4 * hdesc[i].mx * hdesc[i].my);
        dim3 g((maxn + kThreads - 1) / kThreads, (unsigned)ic_list.size());
        if (g.x > 64) g.x = 64;
        mark(0, false);
        k_influence<<<g, kThreads, 0, stream>>>(ddesc, d_ic);
        mark(0, true);
        g_launches += 1;
        if (!ic_single.empty()) {
            for (int i : ic_single) smax = std::max(smax, smem_of(i));
            mark(1, false);
            k_spectra<<<(unsigned)ic_single.size(), kThreads, smax, stream>>>(ddesc, d_ics, 0);
            mark(1, true);
            g_launches += 1;
        }
    }
    // one launch per shared-memory class (requirement within 25% of the class's first, largest
    // member); the classes run concurrently on side streams so that the SMs freed by one class
    // take CTAs of the others instead of idling until the slowest patch of a class finishes
    std::vector<std::pair<int, int>> classes;
    for (int start = 0; start < nsingle;) {
        const size_t sm0 = smem_of(order[start]);
        int end = start + 1;
        while (end < nsingle && smem_of(order[end]) * 5 >= sm0 * 4) end++;
        classes.push_back({start, end});
        start = end;
    }
    mark(2, false);
    if (!classes.empty()) {
        SideStreams &ss = side_streams();
        if (!ss.ok) return (int)cudaErrorNotReady;
        if ((e = cudaEventRecord(ss.fork, stream)) != cudaSuccess) return (int)e;
        for (size_t c = 0; c < classes.size(); c++) {
            cudaStream_t sc = ss.s[c % SideStreams::kN];
            if (c < (size_t)SideStreams::kN && (e = cudaStreamWaitEvent(sc, ss.fork, 0)) != cudaSuccess) return (int)e;
            const int start = classes[c].first, cnt = classes[c].second - classes[c].first;
            const size_t sm0 = smem_of(order[start]);
            k_solve<<<cnt, kThreads, sm0, sc>>>(ddesc, d_order + start, 0);
            g_launches += 1;
        }
        for (int k = 0; k < SideStreams::kN && k < (int)classes.size(); k++) {
            if ((e = cudaEventRecord(ss.join[k], ss.s[k])) != cudaSuccess) return (int)e;
            if ((e = cudaStreamWaitEvent(stream, ss.join[k], 0)) != cudaSuccess) return (int)e;
        }
    }
    // patch groups: cooperative launches, one patch at a time on the caller's stream after
    // all single-CTA work, so that nothing else of this library shares the SMs with them
    for (int k = nsingle; k < (int)order.size(); k++) {
        const int i = order[k];
        const PatchDesc &h = hdesc[i];
        const size_t sm = smem_of(i);
        if ((e = cudaMemsetAsync(h.gscr, 0, 256, stream)) != cudaSuccess) return (int)e;
        const int *lp = d_order + k;
        int grp = 1;
        void *args[3] = {(void *)&ddesc, (void *)&lp, (void *)&grp};
        if (compute_ic[i]) {
            e = cudaLaunchCooperativeKernel((const void *)k_spectra, dim3(h.nblk), dim3(kThreads), args, sm, stream);
            if (e != cudaSuccess) return (int)e;
            if ((e = cudaMemsetAsync(h.gscr, 0, 256, stream)) != cudaSuccess) return (int)e;
            g_launches += 1;
        }
        e = cudaLaunchCooperativeKernel((const void *)k_solve, dim3(h.nblk), dim3(kThreads), args, sm, stream);
        if (e != cudaSuccess) return (int)e;
        g_launches += 1;
    }
    mark(2, true);
    return (int)cudaGetLastError();
}

} // namespace cgb
