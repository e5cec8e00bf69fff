// Device-resident solve of one contact patch by one thread block: set-up of the
// right-hand sides and initial estimate (m_sdis.f90), NORM + NormCG (m_snorm.f90:31-378,
// m_solvpn.f90:24-461), TANG (m_stang.f90:28-951) with the solvers SteadyGS
// (m_solvpt.f90:2825-3254), GDsteady (gdsteady.f90) and TangCG (m_solvpt.f90:1841-2442),
// and the output quantities of soutpt (m_soutpt.f90:377-511).
//
// Every vector operation is a block-strided loop over the npot elements; every scalar
// decision comes from a deterministic block reduction, so all threads follow the same
// control flow.  Products with the influence-coefficient matrix use the FFT convolution of
// fft.cuh in precision T (double, or float in the first phase of the mixed-precision form).
#pragma once
#include "common.cuh"
#include "engine.h"
#include "fft.cuh"

namespace cgb {

constexpr int kMaxLs = 99;   // perform_linesearch max_j, gdsteady.f90:1063

struct SolverSmem {
    RedSmem red;
    // line search table (1-based like the reference)
    double tbl_alpha[kMaxLs + 2], tbl_rho[kMaxLs + 2], tbl_drhoda[kMaxLs + 2];
    double alpha_j;
    int stop_j, nobracket, jcount;
    // generic broadcast slots
    double bd[8];
    int bi[8];
    // phase timers (SM cycles), indexed like O_T_TOTAL .. O_T_CONV32
    long long t[kNumPhaseTimers];
    double algb;      // algorithmic bytes of the convolutions so far
};

// thread 0 accumulates the cycles between a start mark and the end of a phase
#define PHASE_START(v) long long v = clock64()
#define PHASE_END(P, k, v) do { if (threadIdx.x == 0) (P).sm->t[(k)] += clock64() - (v); } while (0)

// view of one patch's memory
struct PView {
    const PatchDesc *d;
    int mx, my, n;
    SolverSmem *sm;
    __device__ double *c(int k) const {
        return k < kIoCols ? d->io + (size_t)k * n : d->wk + (size_t)(k - kIoCols) * n;
    }
    __device__ int *ci(int k) const {
        return k == I_IGS ? igs() : d->wki + (size_t)(k - 1) * n;
    }
    __device__ int *igs() const { return (int *)(d->io + (size_t)kIoCols * n + O_NSCAL); }
    __device__ double *out() const { return d->io + (size_t)kIoCols * n; }
    // float columns 0..17 inside the double columns W_FLS .. W_FLS + 8
    __device__ float *f(int k) const { return (float *)c(W_FLS) + (size_t)k * n; }
};

// strided loop of the patch group over n elements
#define FOR_I(i, n) for (int i = gtid(); i < (n); i += gstride())
// loop of the patch group over the rows of the grid, one row per thread.  Rows go round the
// CTAs first (row iy to CTA iy mod nblk), so that the sequential row scans of a patch group
// spread over all its SMs; for one CTA this is the plain thread-strided loop.
#define FOR_ROW(iy, my) for (int iy = g_grp.rank + (int)threadIdx.x * g_grp.nblk; iy < (my); iy += gstride())

// ------------------------------------------------------------------------------------------
// small helpers
// ------------------------------------------------------------------------------------------
__device__ inline double dsign(double a, double b) { return b >= 0.0 ? fabs(a) : -fabs(a); }
__device__ inline double inv_sqrt(double x) { return rsqrt(x); }
__device__ inline float inv_sqrt(float x) { return rsqrtf(x); }

// unit direction of the tangential traction p/|p| (one reciprocal square root), standing for
// (cos, sin) of atan2(py, px); the reference's direction for p = 0
template <typename R>
__device__ inline void unit_dir(R px, R py, R &nx, R &ny) {
    const R r2 = px * px + py * py;
    if (r2 > R(0)) { const R ri = inv_sqrt(r2); nx = px * ri; ny = py * ri; }
    else { nx = (px < R(0) || (px == R(0) && signbit(px))) ? R(-1) : R(1); ny = R(0); if (signbit(py) && px == R(0)) nx = R(1); }
}

__device__ __noinline__ void count_eldiv(const PView &P, int &nadh, int &nslip, int &nplast, int &nexter) {
    const int *igs = P.igs();
    int v[4] = {0, 0, 0, 0};
    FOR_I(i, P.n) {
        int e = igs[i];
        if (e == Adhes) v[0]++; else if (e == Slip) v[1]++; else if (e == Plast) v[2]++; else v[3]++;
    }
    block_sumi<4>(P.sm->red, v);
    nadh = v[0]; nslip = v[1]; nplast = v[2]; nexter = v[3];
}

// row extents of the interior elements (Areas, m_gridfunc.f90:582-637), 1-based like the
// reference: first = nx, last = 0 for empty rows.  Stored in int column I_EXT: row1st at
// [iy], rowlst at [my + iy].
__device__ __noinline__ void areas(const PView &P) {
    const int mx = P.mx, my = P.my;
    const int *igs = P.igs();
    int *ext = P.ci(I_EXT);
    gsync();
    FOR_ROW(iy, my) {
        const int i0 = iy * mx;
        int first = 1;
        while (igs[(first - 1) + i0] <= Exter && first != mx) first++;
        int last = 0;
        for (int ix = first; ix <= mx; ix++) if (igs[(ix - 1) + i0] >= Adhes) last = ix;
        ext[iy] = first;
        ext[my + iy] = last;
    }
    gsync();
}

// one row of A times a vector restricted to the row extents (gf3_AijPj, m_aijpj.f90:99-254):
// returns sum over blocks (ik,jk) listed in blks/vecs for element ii, times ga_inv.
// blk codes: 0 xx, 1 xy, 2 yy, 3 zz (xy == yx).  vec == nullptr means a vector of ones.
__device__ __noinline__ void direct_rowsum(const PView &P, int ii, int nterm, const int *blks, const double *const *vecs,
                                     double *res /* nres */, const int *resid, int nres) {
    const PatchDesc &d = *P.d;
    const int mx = P.mx, my = P.my;
    const int ix = ii % mx + 1, iy = ii / mx + 1;
    const int *ext = P.ci(I_EXT);
    const size_t bsz = (size_t)4 * mx * my;
    double acc[2] = {0.0, 0.0};
    // iterate over (jy, jx) pairs; each thread takes a strided subset of the flattened range
    for (int jy = 1; jy <= my; jy++) {
        const int j0 = max(1, ext[jy - 1] - 1), j1 = min(mx, ext[my + jy - 1] + 1);
        for (int jx = j0 + gtid(); jx <= j1; jx += gstride()) {
            const size_t off = (size_t)(ix - jx + mx) + (size_t)(iy - jy + my) * 2 * mx;
            const int jj = (jx - 1) + (jy - 1) * mx;
            for (int t = 0; t < nterm; t++) {
                const double c = d.cf[blks[t] * bsz + off];
                const double v = vecs[t] ? vecs[t][jj] : 1.0;
                acc[resid[t]] += c * v;
            }
        }
    }
    if (nres == 1) {
        double s = block_sum1(P.sm->red, acc[0]);
        res[0] = s / d.ga;
    } else {
        double a2[2] = {acc[0], acc[1]};
        block_sum<2>(P.sm->red, a2);
        res[0] = a2[0] / d.ga; res[1] = a2[1] / d.ga;
    }
}

// ------------------------------------------------------------------------------------------
// products with A.  Spectra K[0..6] = xx, xy, yy, zz and the preconditioners zz, xx, yy;
// K[7..10] the coupling blocks of K != 0.
// ------------------------------------------------------------------------------------------
constexpr int kMaxSpectra = 13;

template <typename T>
struct Ops {
    Conv<T> cv;
    // xx, xy, yy, zz, M_zz, M_xx, M_yy; with K != 0 the imaginary spectra of xz, yz, and in
    // steady rolling the real and imaginary parts of xz and of yz of cs - cv (null when absent)
    const T *K[kMaxSpectra];
};

// normal product out = A_zz in (kind 3) or M in (kind 4)
template <typename T>
__device__ inline void prod_n(const Ops<T> &op, const double *in, double *out, int mode, const int *igs, int kind) {
    convolve<T, double>(op.cv, in, nullptr, out, nullptr, 1, op.K[kind], nullptr, nullptr, mode, igs);
}
// coupling products (K != 0), FP64: (outx, outy) = A_tz in through the xz, yz blocks of cs
// (imaginary spectra K[7], K[8]; csv false) or, in steady rolling, of cs - cv (complex spectra
// K[9], K[10] and K[11], K[12]; csv true); or out (+)= A_zt (inx, iny) = -(xz inx + yz iny)
__device__ inline void prod_tz(const Ops<double> &op, const double *in, double *ox, double *oy, int mode,
                               const int *igs, bool csv) {
    if (!csv) {
        convolve<double, double>(op.cv, in, nullptr, ox, nullptr, 1, op.K[7], nullptr, nullptr, mode, igs, 1);
        convolve<double, double>(op.cv, in, nullptr, oy, nullptr, 1, op.K[8], nullptr, nullptr, mode, igs, 2);
    } else {
        convolve<double, double>(op.cv, in, nullptr, ox, nullptr, 1, op.K[9], op.K[10], nullptr, mode, igs, 3);
        convolve<double, double>(op.cv, in, nullptr, oy, nullptr, 1, op.K[11], op.K[12], nullptr, mode, igs, 4);
    }
}
__device__ inline void prod_zt(const Ops<double> &op, const double *inx, const double *iny, double *out, bool add,
                               const int *igs) {
    convolve<double, double>(op.cv, inx, nullptr, out, nullptr, 1, op.K[7], nullptr, nullptr,
                             add ? OUT_ADDINT : OUT_ALL, igs, 1, -1.0);
    convolve<double, double>(op.cv, iny, nullptr, out, nullptr, 1, op.K[8], nullptr, nullptr,
                             add ? OUT_ADDINT : OUT_ADDALL, igs, 2, -1.0);
}
// tangential product (outx, outy) = A_tt (inx, iny)
template <typename T, typename IO = double>
__device__ inline void prod_t(const Ops<T> &op, const IO *inx, const IO *iny, IO *ox, IO *oy, int mode, const int *igs) {
    convolve<T, IO>(op.cv, inx, iny, ox, oy, 2, op.K[0], op.K[1], op.K[2], mode, igs);
}

// ------------------------------------------------------------------------------------------
// NormCG, m_solvpn.f90:24-461.  Returns itcg, or -1 when the reference would abort.
// ------------------------------------------------------------------------------------------
// norm: the N digit of this solve (0 approach prescribed, 1 total force); p0 (sensitivity
// solve, m_solvpn.f90:92-97, 281-290): the tolerance is relative to the change from p0
template <typename T>
__device__ __noinline__ int normcg(const PView &P, const Ops<T> &op, int maxcg, double eps, double &pen, double &err,
                      int &nconv, int norm, const double *p0 = nullptr) {
    const PatchDesc &d = *P.d;
    const int n = P.n;
    RedSmem &red = P.sm->red;
    int *igs = P.igs();
    double *pn = P.c(W_PN), *hstot = P.c(W_HSTOT), *rhs = P.c(W_RHS), *res = P.c(W_RES), *rprv = P.c(W_RPRV);
    double *dd = P.c(W_DD), *z = P.c(W_Z), *v = P.c(W_V), *q = P.c(W_Q);
    const double dxdy = d.dxdy, fntrue = d.fntrue;
    const int numinn = (n <= 150) ? 3 : (n <= 400) ? 2 : 1;
    if (norm == 1) pen = 0.0;
    FOR_I(i, n) { rhs[i] = pen - hstot[i]; }
    double davg = 0.0;
    int ncon = 0;
    { int c = 0; FOR_I(i, n) if (igs[i] >= Adhes) c++; ncon = block_sumi1(red, c); }
    if (norm == 0) {
        double hmin = 1e20; FOR_I(i, n) hmin = fmin(hmin, hstot[i]);
        hmin = block_min1(red, hmin) - pen;
        if (hmin >= 0.0) {
            FOR_I(i, n) { pn[i] = 0.0; igs[i] = Exter; }
            gsync();
            err = 0.0;
            return 0;
        }
    } else {
        if (ncon <= 0) {
            double hmin = 1e20, hmax = -1e20;
            FOR_I(i, n) { hmin = fmin(hmin, hstot[i]); hmax = fmax(hmax, hstot[i]); }
            hmin = block_min1(red, hmin); hmax = block_max1(red, hmax);
            double htrsh = hmin + 0.1 * fmax(hmax - hmin, 1e-10);
            int c = 0;
            FOR_I(i, n) if (hstot[i] < htrsh) { igs[i] = Adhes; c++; }
            ncon += block_sumi1(red, c);
        }
        double s = 0; FOR_I(i, n) s += pn[i];
        double fk = dxdy * block_sum1(red, s);
        if (fabs(fk) < (double)1e-3f * fntrue) {
            double pval = fntrue / (dxdy * (double)(float)ncon);
            FOR_I(i, n) if (igs[i] >= Adhes) pn[i] = pval;
        } else {
            FOR_I(i, n) if (igs[i] >= Adhes) pn[i] *= fntrue / fk;
        }
    }
    // res = rhs - A ps on AllInt, then proj_avg
    prod_n<T>(op, pn, res, OUT_INT, igs, 3); nconv++;
    {
        double s = 0; int c = 0;
        FOR_I(i, n) if (igs[i] >= Adhes) { res[i] = rhs[i] - res[i]; s += res[i]; c++; }
        if (norm == 1) {
            double a[1] = {s}; block_sum<1>(red, a); int cc = block_sumi1(red, c);
            double avg = a[0] / (double)(float)max(1, cc);
            FOR_I(i, n) if (igs[i] >= Adhes) res[i] -= avg;
        }
    }
    gsync();
    double rz1 = 0, rz2 = 0, rms_upd1 = 0, alpha = 0;
    int itcg = 0, itinn = 0;
    double rms_xk = 1.0, rms_upd = 2.0 * eps * rms_xk;
    bool lchanged = false;
    while ((lchanged || rms_upd > eps * rms_xk) && itcg < maxcg) {
        itcg++; itinn++;
        prod_n<T>(op, res, z, OUT_INT, igs, 4); nconv++;
        if (norm == 1) {
            double s = 0; int c = 0;
            FOR_I(i, n) if (igs[i] >= Adhes) { s += z[i]; c++; }
            s = block_sum1(red, s); c = block_sumi1(red, c);
            double avg = s / (double)(float)max(1, c);
            FOR_I(i, n) if (igs[i] >= Adhes) z[i] -= avg;
            gsync();
        }
        rz1 = rz2;
        {
            double a[2] = {0, 0};
            FOR_I(i, n) if (igs[i] >= Adhes) { a[0] += z[i] * res[i]; a[1] += z[i] * rprv[i]; }
            block_sum<2>(red, a);
            rz2 = a[0];
            if (itcg <= 1 || rz1 < 1e-20) {
                FOR_I(i, n) if (igs[i] >= Adhes) v[i] = z[i];
            } else {
                double beta = fmax(0.0, (rz2 - a[1]) / fmax(1e-20, rz1));
                FOR_I(i, n) if (igs[i] >= Adhes) v[i] = beta * v[i] + z[i];
            }
        }
        if (norm == 1) {
            double s = 0; int c = 0;
            FOR_I(i, n) if (igs[i] >= Adhes) { s += v[i]; c++; }
            s = block_sum1(red, s); c = block_sumi1(red, c);
            double avg = s / (double)(float)max(1, c);
            FOR_I(i, n) if (igs[i] >= Adhes) v[i] -= avg;
        }
        prod_n<T>(op, v, q, OUT_INT, igs, 3); nconv++;
        if (norm == 1) {
            double s = 0; int c = 0;
            FOR_I(i, n) if (igs[i] >= Adhes) { s += q[i]; c++; }
            s = block_sum1(red, s); c = block_sumi1(red, c);
            double avg = s / (double)(float)max(1, c);
            FOR_I(i, n) if (igs[i] >= Adhes) q[i] -= avg;
            gsync();
        }
        double rv, vav;
        {
            double a[2] = {0, 0};
            FOR_I(i, n) if (igs[i] >= Adhes) { a[0] += res[i] * v[i]; a[1] += q[i] * v[i]; }
            block_sum<2>(red, a);
            rv = a[0]; vav = a[1];
        }
        if (fabs(vav) > 1e-32 && ncon == 1) alpha = rv / vav;
        else alpha = rv / fmax(1e-20, vav);
        {
            double a[2] = {0, 0};
            FOR_I(i, n) if (igs[i] >= Adhes) {
                pn[i] += alpha * v[i];
                a[0] += v[i] * v[i];
                const double e = p0 ? pn[i] - p0[i] : pn[i];
                a[1] += e * e;
            }
            int c = 0; FOR_I(i, n) if (igs[i] >= Adhes) c++;
            block_sum<2>(red, a);
            c = block_sumi1(red, c);
            rms_upd = fabs(alpha) * sqrt(a[0] / max(1, c));
            if (itcg == 1) rms_upd1 = rms_upd;
            if (itcg <= 3 || itcg % 10 == 0) rms_xk = sqrt(a[1] / max(1, c));
        }
        FOR_I(i, n) rprv[i] = res[i];
        if (itinn < numinn && rms_upd >= eps * rms_xk) {
            FOR_I(i, n) if (igs[i] >= Adhes) res[i] -= alpha * q[i];
            gsync();
        } else {
            int chg = 0, dn = 0;
            FOR_I(i, n) if (igs[i] >= Adhes && pn[i] < 0.0) { igs[i] = Exter; pn[i] = 0.0; chg = 1; dn++; }
            {
                int a[2] = {chg, dn}; block_sumi<2>(red, a);
                chg = a[0]; ncon -= a[1];
            }
            bool lchg_negpn = chg > 0;
            if (ncon <= 0) {
                double hmin = 1e20; FOR_I(i, n) hmin = fmin(hmin, hstot[i]);
                hmin = block_min1(red, hmin);
                int c = 0;
                FOR_I(i, n) if (hstot[i] <= hmin + 1e-5) { igs[i] = Adhes; pn[i] = 0.0; c++; }
                c = block_sumi1(red, c);
                ncon += c;
                if (c > 0) lchg_negpn = true;
            }
            if (norm == 1 && lchg_negpn) {
                double s = 0; FOR_I(i, n) s += pn[i];
                double fk = dxdy * block_sum1(red, s);
                if (fabs(fk) < (double)1e-3f * fntrue) {
                    FOR_I(i, n) if (igs[i] >= Adhes) pn[i] = 1.0;
                    s = 0; FOR_I(i, n) s += pn[i];
                    fk = block_sum1(red, s);
                }
                FOR_I(i, n) if (igs[i] >= Adhes) pn[i] *= fntrue / fk;
            }
            // dd = A ps - rhs on all elements
            prod_n<T>(op, pn, dd, OUT_ALL, igs, 3); nconv++;
            FOR_I(i, n) dd[i] -= rhs[i];
            if (norm == 1) {
                double s = 0; FOR_I(i, n) if (igs[i] >= Adhes) s += dd[i];
                s = block_sum1(red, s);
                davg = s / (double)(float)ncon;
                FOR_I(i, n) if (igs[i] >= Adhes) dd[i] -= davg;   // proj_avg over AllInt (count = ncon)
            }
            gsync();
            int nin = 0;
            FOR_I(i, n) {
                res[i] = (igs[i] >= Adhes) ? -dd[i] : 0.0;
                if (igs[i] == Exter && dd[i] - davg < 0.0) {
                    igs[i] = Adhes; res[i] = -(dd[i] - davg); nin++;
                }
                if (igs[i] == Exter) v[i] = 0.0;
            }
            nin = block_sumi1(red, nin);
            ncon += nin;
            itinn = 0;
            lchanged = (nin > 0) || lchg_negpn;
        }
    }
    if (norm == 1) pen = davg;
    double conv = 1.0;
    if (rms_upd * rms_upd1 > 0.0 && itcg > 1) conv = exp(log(rms_upd / rms_upd1) / (itcg - 1));
    err = rms_upd;
    if (rms_upd > rms_xk && conv > 1.0 && itcg >= maxcg) return -1;
    return itcg;
}

// ------------------------------------------------------------------------------------------
// snorm, m_snorm.f90:31-378.  Returns itnorm (-1 maxin, -2 NormCG divergence).
// ------------------------------------------------------------------------------------------
// htang (K != 0): the normal displacement A_zt p_t of the current tangential tractions, added to
// the undeformed distance (m_snorm.f90:31-378)
template <typename T>
__device__ __noinline__ int snorm(const PView &P, const Ops<T> &op, int maxgs, int maxin, double eps, double &pen,
                     int &itcg_out, int &nconv, const double *htang = nullptr) {
    const int n = P.n, mx = P.mx, my = P.my;
    RedSmem &red = P.sm->red;
    int *igs = P.igs();
    double *pn = P.c(W_PN), *hstot = P.c(W_HSTOT), *h = P.c(W_H), *unn = P.c(W_DD), *one = P.c(W_ONE);
    FOR_I(i, n) { hstot[i] = htang ? h[i] + htang[i] : h[i]; one[i] = 1.0; }
    int itnorm = 0, itcg = 0;
    bool zready;
    do {
        itnorm++;
        zready = true;
        FOR_I(i, n) if (igs[i] < Adhes) pn[i] = 0.0;
        gsync();
        double errpn;
        int it = normcg<T>(P, op, maxgs, eps, pen, errpn, nconv, P.d->norm);
        if (it < 0) { itcg_out = itcg; return -2; }
        itcg += it;
        int newext = 0;
        FOR_I(i, n) if (igs[i] >= Adhes && pn[i] < -errpn) { igs[i] = Exter; pn[i] = 0.0; newext++; }
        newext = block_sumi1(red, newext);
        if (newext > 0) zready = false;
        if (zready) {
            areas(P);
            prod_n<T>(op, pn, unn, OUT_ALL, igs, 3); nconv++;
            int ixc = max(1, mx / 2), iyc = max(1, my / 2);
            int iic = (ixc - 1) + (iyc - 1) * mx;
            int blk[1] = {3}; const double *vv[1] = {nullptr}; int rid[1] = {0}; double tolv[1];
            direct_rowsum(P, iic, 1, blk, vv, tolv, rid, 1);
            double tol = fabs(errpn * tolv[0]);
            int newcon = 0;
            FOR_I(i, n) {
                if (igs[i] == Exter && hstot[i] - pen < 0.0) {
                    double dd = hstot[i] - pen + unn[i];
                    if (dd < -tol) { igs[i] = Adhes; newcon++; }
                }
            }
            newcon = block_sumi1(red, newcon);
            if (newcon != 0) zready = false;
        }
        if (it >= maxgs) zready = false;
    } while (!zready && itnorm < maxin);
    if (!zready) itnorm = -1;
    FOR_I(i, n) if (pn[i] < 0.0 && igs[i] >= Adhes) { pn[i] = 0.0; igs[i] = Exter; }
    gsync();
    itcg_out = itcg;
    return itnorm;
}

// ------------------------------------------------------------------------------------------
// single-element solver plstrc for an elastic element (m_solvpt.f90:3278-3807, no plasticity;
// the plastic trial of the reference cannot succeed there and leaves the element in adhesion)
// ------------------------------------------------------------------------------------------
// kF32Start (the mixed-precision SteadyGS): the slip Newton-Raphson first runs in FP32 from the
// reference's starting point to FP32 accuracy, and the FP64 iteration continues from there with
// the reference's stopping rule (one or two FP64 steps instead of several); detinv_pre, when
// non-zero, is the element's 1 / det(coef), evaluated once per column offset by the caller.
template <typename R, bool kF32Start = false>
__device__ __noinline__ void elm_solve(int &el, const R coef[2][2], R eps, R omegah, R omegas, R pr[3], R mus, R s[2],
                                       R detinv_pre = R(0)) {
    const int maxnr = 10;
    const R prc = R(0.0001);
    const R taucs = R(1e20);
    const R zero = R(0), two = R(2);
    R pold1 = pr[0], pold2 = pr[1];
    R si0[2], si[2] = {zero, zero}, dp[2], fk[2], gradf[2][2];
    si0[0] = s[0] - coef[0][0] * pr[0] - coef[0][1] * pr[1];
    si0[1] = s[1] - coef[1][0] * pr[0] - coef[1][1] * pr[1];
    int itry = 0, violat = 1;
    R trc_bound = zero;
    while (itry <= 3 && violat == 1) {
        itry++;
        if (el == Adhes) {
            trc_bound = mus * pr[2];
            const R detinv =
                detinv_pre != R(0) ? detinv_pre : R(1) / (coef[0][0] * coef[1][1] - coef[0][1] * coef[1][0]);
            dp[0] = (-coef[1][1] * s[0] + coef[0][1] * s[1]) * detinv;
            dp[1] = (coef[1][0] * s[0] - coef[0][0] * s[1]) * detinv;
            pr[0] = pold1 + omegah * dp[0];
            pr[1] = pold2 + omegah * dp[1];
            R pabs2 = sqrt(pr[0] * pr[0] + pr[1] * pr[1]);
            R bnd = fmin(trc_bound, taucs);
            if (pabs2 <= bnd) violat = 0;
            else {
                R pabs1 = sqrt((pold1 + dp[0]) * (pold1 + dp[0]) + (pold2 + dp[1]) * (pold2 + dp[1]));
                if (pabs1 <= bnd) { pr[0] = pr[0] * bnd / pabs2; pr[1] = pr[1] * bnd / pabs2; violat = 0; }
                else violat = 1;
            }
            si[0] = si0[0] + coef[0][0] * pr[0] + coef[0][1] * pr[1];
            si[1] = si0[1] + coef[1][0] * pr[0] + coef[1][1] * pr[1];
        } else if (el == Slip) {
            violat = 0;
            trc_bound = mus * pr[2];
            bool start = false;
            if constexpr (kF32Start) {
                const float c00 = (float)coef[0][0], c01 = (float)coef[0][1], c10 = (float)coef[1][0],
                            c11 = (float)coef[1][1];
                const float t0 = (float)si0[0], t1 = (float)si0[1], tb = (float)trc_bound;
                const float sa = sqrtf(t0 * t0 + t1 * t1);
                float qx = -tb * t0 / sa, qy = -tb * t1 / sa;
                for (int it = 0; it < maxnr; it++) {
                    const float ux = t0 + c00 * qx + c01 * qy, uy = t1 + c10 * qx + c11 * qy;
                    const float g0 = qy * ux - qx * uy, g1 = qx * qx + qy * qy - tb * tb;
                    const float a00 = -2.f * c10 * qx - t1 + (c00 - c11) * qy;
                    const float a01 = 2.f * c01 * qy + t0 + (c00 - c11) * qx;
                    const float a10 = 2.f * qx, a11 = 2.f * qy;
                    const float det = a00 * a11 - a01 * a10;
                    if (det == 0.f) break;
                    const float rd = 1.f / det;
                    const float ex = -(a11 * g0 - a01 * g1) * rd, ey = -(-a10 * g0 + a00 * g1) * rd;
                    qx += ex; qy += ey;
                    if (fabsf(ex) + fabsf(ey) <= 1e-6f * tb) break;
                }
                if (isfinite(qx) && isfinite(qy)) { pr[0] = (R)qx; pr[1] = (R)qy; start = true; }
            }
            if (!start) {
                R sabs = sqrt(si0[0] * si0[0] + si0[1] * si0[1]);
                pr[0] = -trc_bound * si0[0] / sabs;
                pr[1] = -trc_bound * si0[1] / sabs;
            }
            si[0] = si0[0] + coef[0][0] * pr[0] + coef[0][1] * pr[1];
            si[1] = si0[1] + coef[1][0] * pr[0] + coef[1][1] * pr[1];
            fk[0] = pr[1] * si[0] - pr[0] * si[1];
            fk[1] = pr[0] * pr[0] + pr[1] * pr[1] - trc_bound * trc_bound;
            int itnr = 0;
            while (itnr == 0 || (itnr < maxnr && fabs(fk[0]) + fabs(fk[1]) >= prc * eps * trc_bound)) {
                itnr++;
                gradf[0][0] = -two * coef[1][0] * pr[0] - si0[1] + (coef[0][0] - coef[1][1]) * pr[1];
                gradf[0][1] = two * coef[0][1] * pr[1] + si0[0] + (coef[0][0] - coef[1][1]) * pr[0];
                gradf[1][0] = two * pr[0];
                gradf[1][1] = two * pr[1];
                R det = gradf[0][0] * gradf[1][1] - gradf[0][1] * gradf[1][0];
                if (det == zero) itnr = maxnr;
                else {
                    const R rdet = R(1) / det;
                    dp[0] = -(gradf[1][1] * fk[0] - gradf[0][1] * fk[1]) * rdet;
                    dp[1] = -(-gradf[1][0] * fk[0] + gradf[0][0] * fk[1]) * rdet;
                    pr[0] += dp[0]; pr[1] += dp[1];
                }
                si[0] = si0[0] + coef[0][0] * pr[0] + coef[0][1] * pr[1];
                si[1] = si0[1] + coef[1][0] * pr[0] + coef[1][1] * pr[1];
                fk[0] = pr[1] * si[0] - pr[0] * si[1];
                fk[1] = pr[0] * pr[0] + pr[1] * pr[1] - trc_bound * trc_bound;
            }
            if (omegas == R(1)) {
                // no under-relaxation of the angle: the rotation below reduces to scaling the
                // Newton result onto the traction bound
                R ux, uy;
                unit_dir<R>(pr[0], pr[1], ux, uy);
                pr[0] = trc_bound * ux;
                pr[1] = trc_bound * uy;
            } else {
                R alph0 = atan2(pold2, pold1);
                R alph1 = atan2(pr[1], pr[0]);
                R dalph = alph1 - alph0;
                const R pi = R(3.14159265358979323846);
                if (dalph < -pi) dalph += two * pi;
                if (dalph > pi) dalph -= two * pi;
                alph1 = alph0 + omegas * dalph;
                R sn, cs;
                sincos(alph1, &sn, &cs);
                pr[0] = trc_bound * cs;
                pr[1] = trc_bound * sn;
            }
            if (fabs(pr[0]) > fabs(pr[1])) { if (pr[0] * si[0] > zero) violat = 1; }
            else { if (pr[1] * si[1] > zero) violat = 1; }
        } else {
            // plastic trial: with an infinite yield limit it is always rejected
            trc_bound = mus * pr[2];
            si[0] = zero; si[1] = zero;
            violat = 1;
        }
        if (itry <= 3 && violat == 1) {
            if (el == Adhes) el = (trc_bound <= taucs) ? Slip : Plast;
            else if (el == Slip) el = Plast;
            else el = Adhes;
        }
    }
    s[0] = si[0]; s[1] = si[1];
}

struct TangState {
    int solver;
    double omegah, omegas;
};

// ------------------------------------------------------------------------------------------
// SteadyGS, m_solvpt.f90:2825-3254: element-by-element Gauss-Seidel in rolling order.
// Each element's shift is a block reduction; thread 0 solves the element and propagates.
// ------------------------------------------------------------------------------------------
// Tangential row sum of SteadyGS: s = ga_inv * sum_j A_t(ii, j) dp(j) over the row extents of
// the contact area (gf3_AijPj's row1st/rowlst rule).  The (jy, jx) pairs of the bounding box
// of all row extents are spread over the whole block so that every thread loads its share of
// coefficients and vectors independently.
struct GsBox { int jy0, jx0, w, cnt; };

// cf3: blocks xx, xy (= yx), yy of the coefficients in the layout of cf (block stride 4 mx my)
__device__ inline void stdygs_rowsum(const PView &P, const GsBox &b, int ii, const double *dpx, const double *dpy,
                                     double s[2], const double *cf3 = nullptr) {
    const PatchDesc &d = *P.d;
    const int mx = P.mx, my = P.my;
    const int ix = ii % mx + 1, iy = ii / mx + 1;
    const int *ext = P.ci(I_EXT);
    const size_t bsz = (size_t)4 * mx * my;
    if (!cf3) cf3 = d.cf;
    const double *cxx = cf3, *cxy = cf3 + bsz, *cyy = cf3 + 2 * bsz;
    double a[2] = {0.0, 0.0};
    for (int k = gtid(); k < b.cnt; k += gstride()) {
        const int jy = b.jy0 + k / b.w, jx = b.jx0 + k % b.w;
        const int j0 = max(1, ext[jy - 1] - 1), j1 = min(mx, ext[my + jy - 1] + 1);
        if (jx < j0 || jx > j1) continue;
        const size_t off = (size_t)(ix - jx + mx) + (size_t)(iy - jy + my) * 2 * mx;
        const int jj = (jx - 1) + (jy - 1) * mx;
        const double vx = dpx[jj], vy = dpy[jj], c01 = cxy[off];
        a[0] += cxx[off] * vx + c01 * vy;
        a[1] += c01 * vx + cyy[off] * vy;
    }
    block_sum<2>(P.sm->red, a);
    s[0] = a[0] / d.ga;
    s[1] = a[1] / d.ga;
}

// bounding box of the row extents of the contact area (row1st - 1 .. rowlst + 1 per row)
__device__ inline GsBox gs_box(const PView &P) {
    const int mx = P.mx, my = P.my;
    const int *ext = P.ci(I_EXT);
    GsBox box;
    if (threadIdx.x == 0) {
        int jy0 = my + 1, jy1 = 0, jx0 = mx + 1, jx1 = 0;
        for (int jy = 1; jy <= my; jy++) {
            const int j0 = max(1, ext[jy - 1] - 1), j1 = min(mx, ext[my + jy - 1] + 1);
            if (j0 > j1) continue;
            jy0 = min(jy0, jy); jy1 = max(jy1, jy);
            jx0 = min(jx0, j0); jx1 = max(jx1, j1);
        }
        P.sm->bi[0] = jy0; P.sm->bi[1] = jx0;
        P.sm->bi[2] = jx1 >= jx0 ? jx1 - jx0 + 1 : 1;
        P.sm->bi[3] = (jy1 >= jy0 && jx1 >= jx0) ? (jy1 - jy0 + 1) * (jx1 - jx0 + 1) : 0;
    }
    gsync();
    box.jy0 = P.sm->bi[0]; box.jx0 = P.sm->bi[1]; box.w = P.sm->bi[2]; box.cnt = P.sm->bi[3];
    gsync();
    return box;
}

// rms over all elements of the tangential tractions, or of their change from p0 (the stopping
// rule of the sensitivity solves, m_solvpt.f90:2893-2899, 3138-3145)
__device__ inline double rms_from(const PView &P, const double *px, const double *py, const double *p0x,
                                  const double *p0y) {
    double a = 0;
    FOR_I(i, P.n) {
        const double ex = p0x ? px[i] - p0x[i] : px[i], ey = p0y ? py[i] - p0y[i] : py[i];
        a += ex * ex + ey * ey;
    }
    a = block_sum1(P.sm->red, a);
    return sqrt(a / (2 * P.n));
}

// FP32 row sum of the change of dp within the current sweep (mixed-precision SteadyGS):
// ga_inv * sum_j A(ii, j) delta(j) over the row extents, coefficients and changes in FP32
// (per-thread sums), combined across the group in FP64
__device__ inline void stdygs_rowsum32(const PView &P, const GsBox &b, int ii, const float *cf32, const float *ddx,
                                       const float *ddy, double s[2]) {
    const PatchDesc &d = *P.d;
    const int mx = P.mx, my = P.my;
    const int ix = ii % mx + 1, iy = ii / mx + 1;
    const int *ext = P.ci(I_EXT);
    const size_t bsz = (size_t)4 * mx * my;
    const float *cxx = cf32, *cxy = cf32 + bsz, *cyy = cf32 + 2 * bsz;
    float a0 = 0.f, a1 = 0.f;
    for (int k = gtid(); k < b.cnt; k += gstride()) {
        const int jy = b.jy0 + k / b.w, jx = b.jx0 + k % b.w;
        const int j0 = max(1, ext[jy - 1] - 1), j1 = min(mx, ext[my + jy - 1] + 1);
        if (jx < j0 || jx > j1) continue;
        const size_t off = (size_t)(ix - jx + mx) + (size_t)(iy - jy + my) * 2 * mx;
        const int jj = (jx - 1) + (jy - 1) * mx;
        const float vx = ddx[jj], vy = ddy[jj], c01 = cxy[off];
        a0 = fmaf(cxx[off], vx, fmaf(c01, vy, a0));
        a1 = fmaf(c01, vx, fmaf(cyy[off], vy, a1));
    }
    double a[2] = {(double)a0, (double)a1};
    block_sum<2>(P.sm->red, a);
    s[0] = a[0] / d.ga;
    s[1] = a[1] / d.ga;
}

constexpr int kGsPad = 16;

// Warp-cooperative SteadyGS element step of the row-blocked form, run by the lead warp for
// element ii (column ix, row iy) with its shift s0, s1 (valid in lane 0, without the rigid
// shift):
//   - the column jx that closes the element's coefficient (the nearest column behind ix whose
//     element is not in adhesion, the trailing column if there is none) by a warp ballot;
//   - the element solve (plstrc) by lane 0 with the coefficients of its column offset ix - jx,
//     taken from the table ctab (the reference's expression, evaluated once per offset);
//   - the carry of the new traction towards the trailing edge through the adhesion elements
//     behind it, up to and including the first element that is not in adhesion (which keeps its
//     traction and absorbs the change in its dp): the carried tractions are FP64 prefix sums of
//     dp over 32 columns at a time; at the first column whose carried traction exceeds its bound
//     the traction is clipped, that column takes a new dp and the sums restart behind it.
// Every change of dp is recorded in the row's FP32 change rd (dp - dp_b).  GB300 charges an
// FP64 instruction per warp whatever the number of active lanes, so the carry costs a few
// warp-wide FP64 instructions per 32 columns instead of several per column.  Returns (lane 0)
// the squared change of the element's traction.
__device__ inline double gs_element_warp(const PView &P, int ii, int ix, int iy, double s0, double s1, double eps,
                                         double omegah, double omegas, const double *ctab, float *rdx, float *rdy,
                                         const double *dbx, const double *dby, int lane) {
    const PatchDesc &d = *P.d;
    const int mx = P.mx;
    const int ixsta = 1;
    int *igs = P.igs();
    double *px = P.c(W_PX), *py = P.c(W_PY);
    const double *pn = P.c(W_PN);
    double *dpx = P.c(W_DPX), *dpy = P.c(W_DPY);
    const double *wsx = P.c(W_WSX), *wsy = P.c(W_WSY);
    double *sx = P.c(W_SX), *sy = P.c(W_SY);
    const double mus = d.fstat;
    const int row0 = (iy - 1) * mx - 1;        // element index of column kx: row0 + kx
    const unsigned all = 0xffffffffu;
    int jx = ixsta;
    for (int base = ix - 1; base >= ixsta; base -= 32) {
        const int kx = base - lane;
        const unsigned b = __ballot_sync(all, kx >= ixsta && igs[row0 + kx] != Adhes);
        if (b) { jx = base - (__ffs(b) - 1); break; }
    }
    double dif2 = 0.0, pxn = 0.0, pyn = 0.0;
    int eln = 0;
    if (lane == 0) {
        const int o = ix - jx;
        double coef[2][2];
        coef[0][0] = ctab[o];
        coef[0][1] = ctab[mx + o];
        coef[1][0] = coef[0][1];
        coef[1][1] = ctab[2 * mx + o];
        double s[2] = {s0 + wsx[ii], s1 + wsy[ii]};
        double pr[3] = {px[ii], py[ii], pn[ii]};
        int el = igs[ii];
        elm_solve<double, true>(el, coef, eps, omegah, omegas, pr, mus, s, ctab[3 * mx + o]);
        igs[ii] = el;
        dif2 = (pr[0] - px[ii]) * (pr[0] - px[ii]) + (pr[1] - py[ii]) * (pr[1] - py[ii]);
        dpx[ii] += pr[0] - px[ii];
        dpy[ii] += pr[1] - py[ii];
        px[ii] = pr[0]; py[ii] = pr[1];
        sx[ii] = s[0]; sy[ii] = s[1];
        rdx[kGsPad + ix - 1] = (float)(dpx[ii] - dbx[ii]);
        rdy[kGsPad + ix - 1] = (float)(dpy[ii] - dby[ii]);
        pxn = pr[0]; pyn = pr[1]; eln = el;
    }
    pxn = __shfl_sync(all, pxn, 0);
    pyn = __shfl_sync(all, pyn, 0);
    eln = __shfl_sync(all, eln, 0);
    __syncwarp();
    int base = ix - 1;
    while (base >= ixsta) {
        const int kx = base - lane;
        const bool valid = kx >= ixsta;
        const int kk = row0 + kx;
        const int ek = valid ? igs[kk] : Exter;
        // the chain: the lanes before the first one that is not in adhesion (or past the edge)
        const unsigned stop = __ballot_sync(all, !valid || ek != Adhes);
        const int e = stop ? __ffs(stop) - 1 : 32;
        const bool chain = lane < e;
        double ax = chain ? dpx[kk] : 0.0, ay = chain ? dpy[kk] : 0.0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const double tx = __shfl_up_sync(all, ax, o), ty = __shfl_up_sync(all, ay, o);
            if (lane >= o) { ax += tx; ay += ty; }
        }
        const double qx = pxn + ax, qy = pyn + ay;
        // traction in front of each lane: the carried traction of the lane before it
        double fx = __shfl_up_sync(all, qx, 1), fy = __shfl_up_sync(all, qy, 1);
        if (lane == 0) { fx = pxn; fy = pyn; }
        double ptbnd = 0.0;
        bool viol = false;
        if (chain) {
            ptbnd = mus * pn[kk];
            viol = qx * qx + qy * qy > ptbnd * ptbnd;
        }
        const unsigned vb = __ballot_sync(all, viol);
        const int v = vb ? __ffs(vb) - 1 : 32;
        if (chain && lane < v) { px[kk] = qx; py[kk] = qy; }
        if (v < e) {
            // clipped to the traction bound (|p| > bound compared in squares)
            double cx = 0.0, cy = 0.0;
            if (lane == v) {
                const double f = ptbnd * inv_sqrt(qx * qx + qy * qy);
                cx = qx * f; cy = qy * f;
                px[kk] = cx; py[kk] = cy;
                dpx[kk] = cx - fx; dpy[kk] = cy - fy;
                rdx[kGsPad + kx - 1] = (float)(dpx[kk] - dbx[kk]);
                rdy[kGsPad + kx - 1] = (float)(dpy[kk] - dby[kk]);
            }
            pxn = __shfl_sync(all, cx, v);
            pyn = __shfl_sync(all, cy, v);
            eln = Adhes;
            base -= v + 1;
            __syncwarp();
            continue;
        }
        if (e < 32) {
            // lane e ends the carry
            const int efront = e == 0 ? eln : Adhes;
            if (lane == e && valid) {
                bool ch = false;
                if (ek == Slip || ek == Plast) { dpx[kk] = px[kk] - fx; dpy[kk] = py[kk] - fy; ch = true; }
                else if (efront >= Adhes) { dpx[kk] = -fx; dpy[kk] = -fy; ch = true; }
                if (ch) {
                    rdx[kGsPad + kx - 1] = (float)(dpx[kk] - dbx[kk]);
                    rdy[kGsPad + kx - 1] = (float)(dpy[kk] - dby[kk]);
                }
            }
            break;
        }
        // all 32 columns in adhesion and within their bounds: on to the next 32
        pxn = __shfl_sync(all, qx, 31);
        pyn = __shfl_sync(all, qy, 31);
        eln = Adhes;
        base -= 32;
        __syncwarp();
    }
    __syncwarp();
    return dif2;
}

// Row-blocked form of the mixed-precision SteadyGS sweep.  An element's shift within a sweep is
// s_b (the FP64 product of dp_b at the start of the sweep) plus A times the change dp - dp_b
// made so far in the sweep.  That change lives in the rows already swept and in the current
// row only, so the shift splits into
//   - the rows above: after a row is finished, its change is applied to an FP32 accumulator of
//     every element of the rows below it (gs_row_update, spread over the whole patch group,
//     register tiles of kGsTile elements along x with a sliding window of coefficients), and
//   - the current row: a sum over that row's change, held in shared memory, by one warp
//     (gs_inrow_sum), with no block-wide barrier per element.
// Both parts are FP32 products of the sweep's change (which tends to zero as the sweep
// converges); they are added to the FP64 s_b in FP64.  Shared memory (the convolution's batch buffer, free between products):
// coefficient row dy = 0 of blocks xx, xy, yy (3 x 2 mx floats) and the current row's change
// (2 x (mx + 2 kGsPad) floats, zero outside the row).
constexpr int kGsTile = 8;

// bytes: ctab (4 mx doubles), c0 (6 mx floats), rdx and rdy (mx + 2 kGsPad floats each)
__host__ __device__ inline size_t gs_rows_smem_bytes(int mx) {
    return (size_t)32 * mx + 4 * ((size_t)6 * mx + 2 * ((size_t)mx + 2 * kGsPad));
}

// (s0, s1) = sum over jx in [j0, j1] of A(ix - jx, 0) dd(jx) (without the factor ga_inv), FP32
// products and sums; lane 0 returns the sum
__device__ inline void gs_inrow_sum(const float *c0, const float *rdx, const float *rdy, int ix, int j0, int j1, int mx,
                                    int lane, float &s0, float &s1) {
    const float *cxx = c0, *cxy = c0 + 2 * mx, *cyy = c0 + 4 * mx;
    float a0 = 0.f, a1 = 0.f;
    for (int jx = j0 + lane; jx <= j1; jx += 32) {
        const int k = ix - jx + mx;
        const float vx = rdx[kGsPad + jx - 1], vy = rdy[kGsPad + jx - 1], c01 = cxy[k];
        a0 = fmaf(cxx[k], vx, fmaf(c01, vy, a0));
        a1 = fmaf(c01, vx, fmaf(cyy[k], vy, a1));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a0 += __shfl_down_sync(0xffffffffu, a0, o);
        a1 += __shfl_down_sync(0xffffffffu, a1, o);
    }
    s0 = a0; s1 = a1;
}

// four coefficients c[k .. k + 3] of one coefficient row (k + q outside [0, kmax] read as 0;
// a float4 load when all four are inside and aligned, which the caller arranges)
__device__ inline float4 gs_coef4(const float *r, int k, int kmax) {
    if (k >= 0 && k + 3 <= kmax) return *reinterpret_cast<const float4 *>(r + k);
    float4 v;
    v.x = (k + 0 >= 0 && k + 0 <= kmax) ? r[k + 0] : 0.f;
    v.y = (k + 1 >= 0 && k + 1 <= kmax) ? r[k + 1] : 0.f;
    v.z = (k + 2 >= 0 && k + 2 <= kmax) ? r[k + 2] : 0.f;
    v.w = (k + 3 >= 0 && k + 3 <= kmax) ? r[k + 3] : 0.f;
    return v;
}

// acc(t) += sum_jx A(t - (jx, iy)) dd(jx) for the elements t of the rows below iy within
// the box, row by row in tiles of kGsTile elements along x.  Per tile the sum runs over jx from
// high to low, so that the coefficient index k = tx - jx + mx rises by one per step and member m
// of the tile reads c[k + m]: the coefficients sit in a window of kGsWin registers per block
// (xx, xy, yy), refilled four at a time (float4 loads) right after their last use.  The loads
// are aligned by starting the sum up to three columns above j1.  Columns outside [j0, j1] carry
// dd = 0 (the zero padding of the row buffer), so their coefficients only need to be finite:
// they are read inside the coefficient row or as zeros.
constexpr int kGsWin = 2 * kGsTile;

__device__ __noinline__ void gs_row_update(const PView &P, const GsBox &box, int iy, int j0, int j1, const float *rdx,
                                           const float *rdy, const float *cf32, float *accx, float *accy) {
    const int mx = P.mx, my = P.my;
    const int *ext = P.ci(I_EXT);
    const size_t bsz = (size_t)4 * mx * my;
    const int jy1 = box.jy0 + box.cnt / max(box.w, 1) - 1;
    if (box.cnt == 0 || iy >= jy1) return;
    const int ntile = (box.w + kGsTile - 1) / kGsTile;
    const int items = (jy1 - iy) * ntile;
    const int kmax = 2 * mx - 1;
    const int m0 = (int)(((uintptr_t)cf32 >> 2) & 3);
    for (int it = gtid(); it < items; it += gstride()) {
        const int ty = iy + 1 + it / ntile;
        const int tx0 = box.jx0 + kGsTile * (it % ntile);
        const int t0 = ext[ty - 1], t1 = ext[my + ty - 1];
        if (t1 < t0 || tx0 > t1 || tx0 + kGsTile - 1 < t0) continue;
        const int rb = (ty - iy + my) * 2 * mx;
        const float *rxx = cf32 + rb, *rxy = cf32 + bsz + rb, *ryy = cf32 + 2 * bsz + rb;
        const int e = (((m0 + rb + tx0 - j1 + mx) % 4) + 4) % 4;
        const int jstart = j1 + e;
        const int nround = (jstart - j0 + kGsWin) / kGsWin;
        int k = tx0 - jstart + mx;
        float wxx[kGsWin], wxy[kGsWin], wyy[kGsWin], a0[kGsTile], a1[kGsTile];
#pragma unroll
        for (int q = 0; q < kGsWin; q += 4) {
            const float4 u = gs_coef4(rxx, k + q, kmax), v = gs_coef4(rxy, k + q, kmax), w = gs_coef4(ryy, k + q, kmax);
            wxx[q] = u.x; wxx[q + 1] = u.y; wxx[q + 2] = u.z; wxx[q + 3] = u.w;
            wxy[q] = v.x; wxy[q + 1] = v.y; wxy[q + 2] = v.z; wxy[q + 3] = v.w;
            wyy[q] = w.x; wyy[q + 1] = w.y; wyy[q + 2] = w.z; wyy[q + 3] = w.w;
        }
#pragma unroll
        for (int m = 0; m < kGsTile; m++) { a0[m] = 0.f; a1[m] = 0.f; }
        const float *vxp = rdx + kGsPad + jstart - 1, *vyp = rdy + kGsPad + jstart - 1;
        for (int r = 0; r < nround; r++) {
#pragma unroll
            for (int s = 0; s < kGsWin; s++) {
                const float vx = vxp[-s], vy = vyp[-s];
#pragma unroll
                for (int m = 0; m < kGsTile; m++) {
                    const int q = (s + m) % kGsWin;
                    a0[m] = fmaf(wxx[q], vx, fmaf(wxy[q], vy, a0[m]));
                    a1[m] = fmaf(wxy[q], vx, fmaf(wyy[q], vy, a1[m]));
                }
                if (s % 4 == 3) {
                    // slots s - 3 .. s (offsets s - 3 .. s) are used for the last time at this
                    // step; they take offsets kGsWin + s - 3 .. kGsWin + s
                    const int q0 = s - 3;
                    const int kk = k + kGsWin + q0;
                    const float4 u = gs_coef4(rxx, kk, kmax), v = gs_coef4(rxy, kk, kmax), w = gs_coef4(ryy, kk, kmax);
                    wxx[q0] = u.x; wxx[q0 + 1] = u.y; wxx[q0 + 2] = u.z; wxx[q0 + 3] = u.w;
                    wxy[q0] = v.x; wxy[q0 + 1] = v.y; wxy[q0 + 2] = v.z; wxy[q0 + 3] = v.w;
                    wyy[q0] = w.x; wyy[q0 + 1] = w.y; wyy[q0 + 2] = w.z; wyy[q0 + 3] = w.w;
                }
            }
            vxp -= kGsWin; vyp -= kGsWin;
            k += kGsWin;
        }
#pragma unroll
        for (int m = 0; m < kGsTile; m++) {
            const int tx = tx0 + m;
            if (tx >= t0 && tx <= t1) {
                const size_t t = (size_t)(tx - 1) + (size_t)(ty - 1) * mx;
                accx[t] += a0[m];
                accy[t] += a1[m];
            }
        }
    }
}

// SteadyGS, m_solvpt.f90:2825-3254.  o64 (mixed precision): each sweep starts from an FP64
// product s_b = A dp_b of the current dp (one FFT convolution); an element's shift within the
// sweep is s_b plus the FP32 product of the change dp - dp_b made so far in the sweep, so that
// the shift keeps FP64 accuracy up to the FP32 rounding of that change.  The mixed form runs
// row-blocked (gs_row_update) when the row buffers fit the convolution's shared batch buffer,
// element-wise (one group-wide row sum per element) otherwise and in the FP64 form.
__device__ __noinline__ int stdygs(const PView &P, double eps, int maxgs, double omegah, double omegas, int &info,
                                   double &err, const Ops<double> *o64 = nullptr, const double *p0x = nullptr,
                                   const double *p0y = nullptr) {
    PHASE_START(tgs);
    const PatchDesc &d = *P.d;
    const int mx = P.mx, my = P.my, n = P.n;
    RedSmem &red = P.sm->red;
    int *igs = P.igs();
    double *px = P.c(W_PX), *py = P.c(W_PY);
    double *dpx = P.c(W_DPX), *dpy = P.c(W_DPY);
    const size_t bsz = (size_t)4 * mx * my;
    const int ixsta = 1, ixinc = 1, ixend = mx;
    const bool mix = o64 != nullptr;
    // mixed: FP32 coefficients xx, xy, yy (6 double columns from W_FST), the FP32 change (one
    // double column after them), the FP64 base dp_b and its product s_b
    float *cf32 = (float *)P.c(W_FST);
    float *ddx = (float *)P.c(W_FST + 6), *ddy = ddx + n;
    double *dbx = P.c(W_DBX), *dby = P.c(W_DBY), *sbx = P.c(W_SBX), *sby = P.c(W_SBY);
    // row-blocked form: FP32 sums of the rows' changes so far in the sweep (column W_TX)
    float *accx = (float *)P.c(W_TX), *accy = accx + n;
    const bool rows = mix && gs_rows_smem_bytes(mx) <= (size_t)o64->cv.ccap * sizeof(C<double>);
    double *ctab = nullptr;
    float *c0 = nullptr, *rdx = nullptr, *rdy = nullptr;
    if (rows) {
        ctab = (double *)o64->cv.cbuf;
        c0 = (float *)(ctab + 4 * mx);
        rdx = c0 + 6 * mx;
        rdy = rdx + mx + 2 * kGsPad;
    }
    if (mix) {
        for (int t = gtid(); t < (int)(3 * bsz); t += gstride()) cf32[t] = (float)d.cf[t];
    }
    FOR_I(ii, n) {
        int ix = ii % mx + 1;
        if (ix != ixend) { dpx[ii] = px[ii] - px[ii + ixinc]; dpy[ii] = py[ii] - py[ii + ixinc]; }
        else { dpx[ii] = px[ii]; dpy[ii] = py[ii]; }
    }
    int nadh, nslip, nplst, nexter;
    count_eldiv(P, nadh, nslip, nplst, nexter);
    int k = nadh + nslip + nplst;
    double facnel = sqrt((double)(float)n / (double)(float)k);
    // bounding box of the row extents (constant: the contact area does not change in TANG)
    const GsBox box = gs_box(P);
    const int *ext = P.ci(I_EXT);
    int itgs = 0;
    double dif = 2.0, difid = 1.0, dif1 = 0.0;
    while (dif >= difid && itgs < maxgs) {
        itgs++;
        if (mix) {
            FOR_I(i, n) { dbx[i] = dpx[i]; dby[i] = dpy[i]; ddx[i] = 0.f; ddy[i] = 0.f; accx[i] = 0.f; accy[i] = 0.f; }
            prod_t<double>(*o64, dbx, dby, sbx, sby, OUT_ALL, igs);
        }
        double difacc = 0.0;      // held by the group's lead thread
        if (rows) {
            // coefficient row dy = 0 in shared memory (the product above used the buffer), and the
            // element coefficients xx, xy, yy per column offset o = ix - jx (1 .. mx - 1) with
            // 1 / det of each offset's 2 x 2 block
            const float *cr = cf32 + (size_t)my * 2 * mx;
            for (int t = threadIdx.x; t < 2 * mx; t += blockDim.x) {
                c0[t] = cr[t]; c0[2 * mx + t] = cr[bsz + t]; c0[4 * mx + t] = cr[2 * bsz + t];
            }
            {
                const size_t o0 = (size_t)(0 + mx) + (size_t)(0 + my) * 2 * mx;
                for (int t = threadIdx.x; t < 3 * mx; t += blockDim.x) {
                    const int c = t / mx, o = t % mx;
                    const size_t oj = (size_t)(-o + mx) + (size_t)(0 + my) * 2 * mx;
                    ctab[t] = o == 0 ? 0.0 : (d.cf[c * bsz + o0] - d.cf[c * bsz + oj]) / d.ga;
                }
                __syncthreads();
                for (int o = threadIdx.x; o < mx; o += blockDim.x)
                    ctab[3 * mx + o] = o == 0 ? 0.0
                                              : 1.0 / (ctab[o] * ctab[2 * mx + o] - ctab[mx + o] * ctab[mx + o]);
            }
            const double gainv = 1.0 / d.ga;
            const bool lead_warp = g_grp.rank == 0 && threadIdx.x < 32;
            const int lane = threadIdx.x & 31;
            for (int iy = 1; iy <= my; iy++) {
                const int j0 = max(1, ext[iy - 1] - 1), j1 = min(mx, ext[my + iy - 1] + 1);
                if (j0 > j1) continue;
                for (int t = threadIdx.x; t < mx + 2 * kGsPad; t += blockDim.x) { rdx[t] = 0.f; rdy[t] = 0.f; }
                __syncthreads();
                if (lead_warp) {
                    const long long tser = clock64();
                    for (int ix = max(j0, ixsta + 1); ix <= j1; ix++) {
                        const int ii = (ix - 1) + (iy - 1) * mx;
                        if (igs[ii] < Adhes) continue;
                        float r0, r1;
                        gs_inrow_sum(c0, rdx, rdy, ix, j0, j1, mx, lane, r0, r1);
                        double s0 = 0.0, s1 = 0.0;
                        if (lane == 0) {
                            s0 = ((double)accx[ii] + (double)r0) * gainv + sbx[ii];
                            s1 = ((double)accy[ii] + (double)r1) * gainv + sby[ii];
                        }
                        difacc += gs_element_warp(P, ii, ix, iy, s0, s1, eps, omegah, omegas, ctab, rdx, rdy, dbx,
                                                  dby, lane);
                    }
                    // a patch group: the row's change goes to the other CTAs through global memory
                    if (g_grp.nblk > 1)
                        for (int jx = j0 + lane; jx <= j1; jx += 32) {
                            const int jj = (jx - 1) + (iy - 1) * mx;
                            ddx[jj] = rdx[kGsPad + jx - 1]; ddy[jj] = rdy[kGsPad + jx - 1];
                        }
                    if (lane == 0) P.sm->t[O_T_GSSER - O_T_TOTAL] += clock64() - tser;
                }
                gsync();
                if (g_grp.nblk > 1 && g_grp.rank != 0) {
                    for (int jx = j0 + (int)threadIdx.x; jx <= j1; jx += blockDim.x) {
                        const int jj = (jx - 1) + (iy - 1) * mx;
                        rdx[kGsPad + jx - 1] = ddx[jj]; rdy[kGsPad + jx - 1] = ddy[jj];
                    }
                    __syncthreads();
                }
                gs_row_update(P, box, iy, j0, j1, rdx, rdy, cf32, accx, accy);
                gsync();
            }
        } else {
            for (int iy = 1; iy <= my; iy++) {
                for (int ix = ixsta; ix <= ixend; ix++) {
                    int ii = (ix - 1) + (iy - 1) * mx;
                    if (igs[ii] < Adhes) continue;
                    double s[2];
                    if (mix) stdygs_rowsum32(P, box, ii, cf32, ddx, ddy, s);
                    else stdygs_rowsum(P, box, ii, dpx, dpy, s);
                    if (glead() && ix > ixsta) {
                        if (mix) { s[0] += sbx[ii]; s[1] += sby[ii]; }
                        double *pn = P.c(W_PN), *sx = P.c(W_SX), *sy = P.c(W_SY);
                        const double *wsx = P.c(W_WSX), *wsy = P.c(W_WSY);
                        const double mus = d.fstat;
                        // the solver choice keeps the trailing column ix = 1 outside the contact area
                        int jx = ix - ixinc;
                        int jj = (jx - 1) + (iy - 1) * mx;
                        while (igs[jj] == Adhes && jx != ixsta) { jx -= ixinc; jj = (jx - 1) + (iy - 1) * mx; }
                        const size_t o0 = (size_t)(0 + mx) + (size_t)(0 + my) * 2 * mx;
                        const size_t oj = (size_t)(jx - ix + mx) + (size_t)(0 + my) * 2 * mx;
                        double coef[2][2];
                        coef[0][0] = (d.cf[0 * bsz + o0] - d.cf[0 * bsz + oj]) / d.ga;
                        coef[0][1] = (d.cf[1 * bsz + o0] - d.cf[1 * bsz + oj]) / d.ga;
                        coef[1][0] = coef[0][1];
                        coef[1][1] = (d.cf[2 * bsz + o0] - d.cf[2 * bsz + oj]) / d.ga;
                        s[0] += wsx[ii]; s[1] += wsy[ii];
                        double pr[3] = {px[ii], py[ii], pn[ii]};
                        int el = igs[ii];
                        elm_solve(el, coef, eps, omegah, omegas, pr, mus, s);
                        igs[ii] = el;
                        difacc += (pr[0] - px[ii]) * (pr[0] - px[ii]) + (pr[1] - py[ii]) * (pr[1] - py[ii]);
                        dpx[ii] += pr[0] - px[ii];
                        dpy[ii] += pr[1] - py[ii];
                        px[ii] = pr[0]; py[ii] = pr[1];
                        sx[ii] = s[0]; sy[ii] = s[1];
                        if (mix) { ddx[ii] = (float)(dpx[ii] - dbx[ii]); ddy[ii] = (float)(dpy[ii] - dby[ii]); }
                        double pxn = px[ii], pyn = py[ii];
                        int eln = igs[ii];
                        for (int kx = ix - ixinc; kx >= ixsta; kx -= ixinc) {
                            const int kk = (kx - 1) + (iy - 1) * mx;
                            const int ek = igs[kk];
                            if (ek == Adhes) {
                                const double qx = pxn + dpx[kk], qy = pyn + dpy[kk];
                                const double pp = qx * qx + qy * qy, ptbnd = mus * pn[kk];
                                if (pp > ptbnd * ptbnd) {
                                    const double f = ptbnd * inv_sqrt(pp);
                                    const double cx = qx * f, cy = qy * f;
                                    px[kk] = cx; py[kk] = cy;
                                    dpx[kk] = cx - pxn; dpy[kk] = cy - pyn;
                                    pxn = cx; pyn = cy;
                                } else {
                                    px[kk] = qx; py[kk] = qy;
                                    pxn = qx; pyn = qy;
                                }
                            } else if (ek == Slip || ek == Plast) {
                                const double cx = px[kk], cy = py[kk];
                                dpx[kk] = cx - pxn; dpy[kk] = cy - pyn;
                            } else if (eln >= Adhes) {
                                dpx[kk] = -pxn; dpy[kk] = -pyn;
                            }
                            if (mix) { ddx[kk] = (float)(dpx[kk] - dbx[kk]); ddy[kk] = (float)(dpy[kk] - dby[kk]); }
                            if (ek != Adhes) break;
                            eln = ek;
                        }
                    }
                    gsync();
                }
            }
        }
        // the lead thread's sum, broadcast to the group (the other threads add zeros)
        dif = sqrt(block_sum1(red, glead() ? difacc : 0.0) / (2.0 * k));
        const double rms = rms_from(P, px, py, p0x, p0y);
        difid = eps * fmax(1e-6, facnel * rms);
        if (itgs == 1) dif1 = dif;
    }
    double conv = 1.0;
    if (dif * dif1 != 0.0 && itgs > 1) conv = exp(log(dif / dif1) / (itgs - 1));
    err = dif;
    info = 0;
    if (itgs >= maxgs) info = 1;
    if (itgs >= maxgs && conv > 0.997) info = 2;
    if (itgs >= maxgs && conv > 1.0) info = 3;
    PHASE_END(P, O_T_GS - O_T_TOTAL, tgs);
    return itgs;
}

// ------------------------------------------------------------------------------------------
// ConvexGS, m_solvpt.f90:2446-2821 (elastic): block Gauss-Seidel over the contact elements in
// index order with the element solver plstrc.  The shift of an element comes from the current
// tractions: through cs for shifts and transient rolling; for steady rolling through
// csv = cs - cv (one rolling step apart, steady_coefs) or, for elements within one rolling
// step of their leading edge (edge[ii] > 0), through cs minus the displacement difference just
// past that edge (subnd, m_leadedge.f90:336-394), refreshed at the start of every sweep.
// Each element's row sum is a group reduction; the group's lead thread solves the element.
// edge: per element the 1-based column of its leading edge, 0 when the element takes no edge
// estimate; csv: blocks xx, xy, yy (steady rolling), else nullptr.
// ------------------------------------------------------------------------------------------
__device__ __noinline__ int cnvxgs(const PView &P, const Ops<double> &op, const double *csv, const int *edge,
                                   bool any_edge, double eps, int maxgs, double omegah, double omegas, int &info,
                                   double &err, const double *p0x = nullptr, const double *p0y = nullptr) {
    PHASE_START(tgs);
    const PatchDesc &d = *P.d;
    const int mx = P.mx, my = P.my, n = P.n;
    RedSmem &red = P.sm->red;
    int *igs = P.igs();
    double *px = P.c(W_PX), *py = P.c(W_PY), *pn = P.c(W_PN);
    const double *wsx = P.c(W_WSX), *wsy = P.c(W_WSY);
    double *sx = P.c(W_SX), *sy = P.c(W_SY);
    double *ux = P.c(W_UX), *uy = P.c(W_UY);       // cs p, for the leading-edge estimate
    const size_t bsz = (size_t)4 * mx * my;
    const size_t o0 = (size_t)mx + (size_t)my * 2 * mx;
    const double mus = d.fstat;
    const bool ssrol = csv != nullptr;
    double coefs[2][2], coefsv[2][2];
    coefs[0][0] = d.cf[0 * bsz + o0] / d.ga; coefs[0][1] = d.cf[1 * bsz + o0] / d.ga;
    coefs[1][0] = coefs[0][1];               coefs[1][1] = d.cf[2 * bsz + o0] / d.ga;
    const double *cv = ssrol ? csv : d.cf;
    coefsv[0][0] = cv[0 * bsz + o0] / d.ga; coefsv[0][1] = cv[1 * bsz + o0] / d.ga;
    coefsv[1][0] = coefsv[0][1];            coefsv[1][1] = cv[2 * bsz + o0] / d.ga;
    int nadh, nslip, nplst, nexter;
    count_eldiv(P, nadh, nslip, nplst, nexter);
    const int k = nadh + nslip + nplst;
    if (k == 0) { info = 0; err = 0.0; PHASE_END(P, O_T_GS - O_T_TOTAL, tgs); return 0; }
    const double facnel = sqrt((double)(float)n / (double)(float)k);
    const GsBox box = gs_box(P);
    int itgs = 0;
    double dif = 2.0, difid = 1.0, dif1 = 0.0;
    while (dif >= difid && itgs < maxgs) {
        itgs++;
        if (ssrol && any_edge) {
            // u = cs p on all elements: the edge estimate of position ix0 is u at ix0 + 1
            // (facdx = 1 for ConvexGS), zero when the edge is within two elements of the end
            prod_t<double>(op, px, py, ux, uy, OUT_ALL, igs);
        }
        double difacc = 0.0;      // held by the group's lead thread
        for (int ii = 0; ii < n; ii++) {
            const int el0 = igs[ii];
            if (el0 < Adhes) continue;
            if (!(itgs <= 1000 || itgs % 2 == 0 || el0 == Adhes)) continue;
            const int ix0 = ssrol ? edge[ii] : 0;
            const bool zledge = ix0 > 0;
            double s[2];
            stdygs_rowsum(P, box, ii, px, py, s, zledge ? d.cf : cv);
            if (glead()) {
                s[0] += wsx[ii]; s[1] += wsy[ii];
                if (zledge && ix0 + 2 <= mx) {
                    const int je = ix0 + (ii / mx) * mx;     // 0-based index of column ix0 + 1
                    s[0] -= ux[je]; s[1] -= uy[je];
                }
                double pr[3] = {px[ii], py[ii], pn[ii]};
                int el = el0;
                elm_solve(el, zledge ? coefs : coefsv, eps, omegah, omegas, pr, mus, s);
                igs[ii] = el;
                difacc += (px[ii] - pr[0]) * (px[ii] - pr[0]) + (py[ii] - pr[1]) * (py[ii] - pr[1]);
                px[ii] = pr[0]; py[ii] = pr[1];
                sx[ii] = s[0]; sy[ii] = s[1];
            }
            gsync();
        }
        dif = sqrt(block_sum1(red, glead() ? difacc : 0.0) / (2.0 * k));
        const double rms = rms_from(P, px, py, p0x, p0y);
        difid = eps * fmax(1e-6, facnel * rms);
        if (itgs == 1) dif1 = dif;
    }
    double conv = 1.0;
    if (dif * dif1 != 0.0 && itgs > 1) conv = exp(log(dif / dif1) / (itgs - 1));
    err = dif;
    info = 0;
    if (itgs >= maxgs) info = 1;
    if (itgs >= maxgs && conv > 0.997) info = 2;
    if (itgs >= maxgs && conv > 1.0) info = 3;
    PHASE_END(P, O_T_GS - O_T_TOTAL, tgs);
    return itgs;
}

// ------------------------------------------------------------------------------------------
// GDsteady helpers (gdsteady.f90:610-1462); rows are scanned from the leading edge (ix = mx)
// towards the trailing edge, one thread per row.
// ------------------------------------------------------------------------------------------
// The row scans below are sequential along x; their loads do not depend on the scan, so
// each thread loads the next kScanBatch elements of its row while it runs the recurrence over
// the current ones (two register buffers): the memory latency overlaps the dependent
// arithmetic instead of adding to it.  The arithmetic is the same, element by element, as a
// plain loop.
template <typename R>
struct ScanBatch { static constexpr int U = sizeof(R) == 8 ? 4 : 8; };

// inputs of the traction-bound scan for elements ixb, ixb-1, ..., ixb-U+1 of row i0: element
// type, increment (dp, or dp + alpha dv in the line search) and bound; zeros past the row start
template <typename R, int U>
struct ScanIn {
    int el[U];
    R ax[U], ay[U], tb[U];
    __device__ __forceinline__ void load(int ixb, int i0, const int *igs, const R *dpx, const R *dpy, const R *dvx,
                                         const R *dvy, R aj, const R *trc) {
#pragma unroll
        for (int u = 0; u < U; u++) {
            const int ii = ixb - u + i0;
            el[u] = Exter; ax[u] = ay[u] = tb[u] = R(0);
            if (ixb - u >= 0) {
                el[u] = igs[ii];
                if (dvx) { ax[u] = dpx[ii] + aj * dvx[ii]; ay[u] = dpy[ii] + aj * dvy[ii]; }
                else { ax[u] = dpx[ii]; ay[u] = dpy[ii]; }
                tb[u] = trc[ii];
            }
        }
    }
};

// one traction-bound step: q = p(ix+1) + increment, clipped to the bound in slip elements
// and where |q| reaches it (apply_trcbnd, gdsteady.f90:807-847)
template <typename R>
__device__ __forceinline__ void trcbnd_step(int el, R ax, R ay, R tb, R pxn, R pyn, R &qx, R &qy) {
    qx = R(0); qy = R(0);
    if (el > Exter) {
        qx = pxn + ax; qy = pyn + ay;
        const R qq = qx * qx + qy * qy;
        if (el == Slip || qq >= tb * tb) { const R f = tb * inv_sqrt(qq); qx *= f; qy *= f; }
    }
}

// traction-bound scan of every row of the group: p from the increments, written to (ox, oy);
// with wdpx/wdpy the clipped increments dp = q - p(ix+1) are written there (they may be the
// input increments: an element is read one batch before it is written)
template <typename R>
__device__ __forceinline__ void trcbnd_rows(const PView &P, const R *trc, const R *dpx, const R *dpy, const R *dvx,
                                            const R *dvy, R aj, R *ox, R *oy, R *wdpx, R *wdpy) {
    const int mx = P.mx, my = P.my;
    const int *igs = P.igs();
    constexpr int U = ScanBatch<R>::U;
    FOR_ROW(iy, my) {
        const int i0 = iy * mx;
        ox[(mx - 1) + i0] = R(0); oy[(mx - 1) + i0] = R(0);
        R pxn = R(0), pyn = R(0);
        ScanIn<R, U> cur, nxt;
        cur.load(mx - 2, i0, igs, dpx, dpy, dvx, dvy, aj, trc);
        for (int ixb = mx - 2; ixb >= 0; ixb -= U) {
            nxt.load(ixb - U, i0, igs, dpx, dpy, dvx, dvy, aj, trc);
#pragma unroll
            for (int u = 0; u < U; u++) {
                if (ixb - u < 0) break;
                const int ii = ixb - u + i0;
                R qx, qy;
                trcbnd_step<R>(cur.el[u], cur.ax[u], cur.ay[u], cur.tb[u], pxn, pyn, qx, qy);
                ox[ii] = qx; oy[ii] = qy;
                if (wdpx) { wdpx[ii] = qx - pxn; wdpy[ii] = qy - pyn; }
                pxn = qx; pyn = qy;
            }
            cur = nxt;
        }
    }
}

template <typename R>
__device__ __noinline__ void apply_trcbnd(const PView &P, const R *trc, R *dpx, R *dpy, R *px, R *py) {
    gsync();
    PHASE_START(tsc);
    trcbnd_rows<R>(P, trc, dpx, dpy, nullptr, nullptr, R(0), px, py, dpx, dpy);
    gsync();
    PHASE_END(P, O_T_SCAN - O_T_TOTAL, tsc);
}

// compute_diagscaling, gdsteady.f90:901-1042.  In the reference 'elnew' and 'fac_s' carry over
// from one element to the next.  The carried values reach (a) exterior elements, whose
// scaling is never used (their residual and line-search terms are zero), and (b) slip
// elements whose angle error stays below tiny_err after the perturbation.  All other
// elements are independent and are handled in parallel; when a case (b) element exists the
// whole pass is repeated serially with the reference's carry-over.
// jx: the last element at or behind ix (towards the trailing edge, 1-based) that is not in
// adhesion, or 1 (the reference's backward search from ix); see trailing_nonadh
template <typename R>
__device__ inline R dscl_adhesion(const PatchDesc &d, int ix, int jx, R old) {
    const R d_cns = (R)d.d_cns, d_ifc = (R)d.d_ifc, d_lin = (R)d.d_lin;
    R dn;
    if (d_cns < d_ifc) dn = fmax(d_cns, d_ifc + R(ix - jx - 1) * fmin(R(0), d_lin));
    else dn = fmin(d_cns, d_ifc + R(ix - jx - 1) * fmax(R(0), d_lin));
    return fmin(R(50) * old, dn);
}

// angle from a to b in (-pi, pi], atan2 of cross and dot product.  For angles below 0.01 rad
// (the usual case near convergence) the odd series of atan in r = cross / dot up to r^7: its
// truncation, r^9 / 9, is below 1.2e-17 of the angle, so the value is that of atan2 to rounding
// at a fraction of its FP64 instructions.
template <typename R>
__device__ inline R vec_angle(R ax, R ay, R bx, R by) {
    const R cr = ax * by - ay * bx, dt = ax * bx + ay * by;
    if constexpr (sizeof(R) == 8) {
        if (dt > 0.0 && fabs(cr) < 0.01 * dt) {
            const double r = cr / dt, r2 = r * r;
            return r * (1.0 - r2 * (1.0 / 3.0 - r2 * (1.0 / 5.0 - r2 * (1.0 / 7.0))));
        }
    }
    return atan2(cr, dt);
}

// x^p of the diagonal scaling.  For the default exponent p = 0.9 and moderate x: an FP32 start
// exp2(0.9 log2 x) refined by two Newton steps on y^10 = x^9 in FP64 (quadratic convergence from
// ~3e-7: the result is x^0.9 to rounding), in place of the FP64 pow; pow otherwise.
template <typename R>
__device__ inline R pow_scaling(R x, R p) {
    if constexpr (sizeof(R) == 8) {
        if (p == 0.9 && x >= 1e-30 && x <= 1e30) {
            const double x2 = x * x, x4 = x2 * x2, c = x4 * x4 * x;
            double y = (double)exp2f(0.9f * log2f((float)x));
            for (int k = 0; k < 2; k++) {
                const double y2 = y * y, y4 = y2 * y2, y9 = y4 * y4 * y, y10 = y9 * y;
                y = y - (y10 - c) / (10.0 * y9);
            }
            return y;
        }
    }
    return pow(x, p);
}

// angle error of a slip element (perturbed once when it is tiny); returns false if it stays tiny
template <typename R>
__device__ inline bool slip_element(const PatchDesc &d, const R coefs[2][2], R px, R py, R pn, R sx, R sy, int &elnew,
                                    R &fac_s) {
    const R tiny_err = R(1e-6), pi = R(3.14159265358979323846), two = R(2);
    const R fstat = (R)d.fstat;
    // angle from a to b in (-pi, pi] (the reference takes the difference of two atan2 values
    // and wraps it)
    auto angle = [](R ax, R ay, R bx, R by) { return vec_angle<R>(ax, ay, bx, by); };
    (void)pi; (void)two;
    R pr[3] = {px, py, pn};
    R si[2] = {sx, sy};
    R err_0 = angle(pr[0], pr[1], -si[0], -si[1]);
    if (fabs(err_0) <= tiny_err) {
        R c, s; sincos(atan2(pr[1], pr[0]) + R(0.1), &s, &c);
        pr[0] = fstat * pr[2] * c;
        pr[1] = fstat * pr[2] * s;
        si[0] = sx + coefs[0][0] * (pr[0] - px) + coefs[0][1] * (pr[1] - py);
        si[1] = sy + coefs[1][0] * (pr[0] - px) + coefs[1][1] * (pr[1] - py);
        err_0 = angle(pr[0], pr[1], -si[0], -si[1]);
    }
    if (fabs(err_0) <= tiny_err) return false;
    const R s0x = -si[0], s0y = -si[1];
    elnew = Slip;
    elm_solve<R>(elnew, coefs, R(1e-6), R(1), R(1), pr, fstat, si);
    if (elnew == Slip) {
        const R upd_s = angle(s0x, s0y, -si[0], -si[1]);
        fac_s = fabs(upd_s) / fabs(err_0);
    }
    return true;
}

// arrays read and written by the line search, in its working precision
template <typename R>
struct LsArrays {
    const R *dpx, *dpy, *dvx, *dvy, *vx, *vy, *qx, *qy, *sx, *sy, *nox, *noy, *dscl, *trc;
    R *pdx, *pdy, *pnx, *pny;
};

// single-precision copies of the line-search inputs, made once per line search
__device__ inline void ls_arrays(const PView &P, LsArrays<float> &A) {
    const int n = P.n;
    const int src[14] = {W_DPX, W_DPY, W_DVX, W_DVY, W_VX, W_VY, W_QX, W_QY, W_SX, W_SY, W_NX, W_NY, W_DSCL, W_TRC};
    const float *f[18];
    for (int k = 0; k < 14; k++) {
        float *dst = P.f(k);
        const double *from = P.c(src[k]);
        FOR_I(i, n) dst[i] = (float)from[i];
        f[k] = dst;
    }
    A.dpx = f[0]; A.dpy = f[1]; A.dvx = f[2]; A.dvy = f[3]; A.vx = f[4]; A.vy = f[5]; A.qx = f[6]; A.qy = f[7];
    A.sx = f[8]; A.sy = f[9]; A.nox = f[10]; A.noy = f[11]; A.dscl = f[12]; A.trc = f[13];
    A.pdx = P.f(14); A.pdy = P.f(15); A.pnx = P.f(16); A.pny = P.f(17);
    gsync();
}

// perform_linesearch, gdsteady.f90:1046-1462.  Evaluations of rho(alpha) are block-parallel;
// the Brent bookkeeping runs on thread 0 with the table in shared memory.
// R = float (mixed precision): the trial tractions and the terms of the merit function are
// evaluated in single precision (sums in double); the step length only has to be found to
// the relative tolerance eps_j = 1e-3 of the bracketing search
template <typename R>
__device__ __noinline__ bool perform_linesearch(const PView &P, const LsArrays<R> &A, double alpha0, double &alpha_out,
                                                int &jout) {
    PHASE_START(tls);
    const int n = P.n;
    SolverSmem &S = *P.sm;
    RedSmem &red = S.red;
    const int *igs = P.igs();
    const double tiny = 1e-12, eps_j = 0.001;
    const R rtiny = R(1e-12);
    // thread-0 state
    int itb_a = 0, itb_b = 0, itb_x = 0, itb_w = 0, itb_v = 0, itb_u = 0;
    double dst_cur = 0, dst_prv1 = 0, dst_prv2 = 0, ddrho = 0, alpha_prv = -1.0;
    bool has_bracket = false;
    int j = 0;
    if (threadIdx.x == 0) { S.alpha_j = 0.0; S.stop_j = 0; S.nobracket = 0; }
    gsync();
    // adhesion elements keep their status during the search and their terms do not depend on
    // the trial tractions: their part of rho is the quadratic qa0 + 2 alpha qa1 + alpha^2 qa2
    double qa[3] = {0.0, 0.0, 0.0};
    {
        FOR_I(ii, n) if (igs[ii] == Adhes) {
            const R d2 = A.dscl[ii] * A.dscl[ii];
            qa[0] += (double)(d2 * (A.sx[ii] * A.sx[ii] + A.sy[ii] * A.sy[ii]));
            qa[1] += (double)(d2 * (A.sx[ii] * A.qx[ii] + A.sy[ii] * A.qy[ii]));
            qa[2] += (double)(d2 * (A.qx[ii] * A.qx[ii] + A.qy[ii] * A.qy[ii]));
        }
        block_sum<3>(red, qa);
    }
    for (int guard = 0; guard < kMaxLs + 1; guard++) {
        const double alpha_j = S.alpha_j;
        const R aj = (R)alpha_j;
        // trial tractions: the traction-bound scan of dp + alpha dv along each row (apply_trcbnd)
        {
            PHASE_START(tsc);
            trcbnd_rows<R>(P, A.trc, A.dpx, A.dpy, A.dvx, A.dvy, aj, A.pnx, A.pny, nullptr, nullptr);
            gsync();
            PHASE_END(P, O_T_SCAN - O_T_TOTAL, tsc);
        }
        double acc[4] = {0, 0, 0, 0};     // rho, c0, c1, c2 of the slip elements
        FOR_I(ii, n) {
            if (igs[ii] != Slip) continue;
            const R txo = -A.noy[ii], tyo = A.nox[ii];
            const R vt = A.vx[ii] * txo + A.vy[ii] * tyo;
            const R tb = A.trc[ii];
            const R dth_da = (tb * vt) / (fmax(rtiny, tb * tb) + aj * aj * vt * vt);
            R nxn, nyn;
            unit_dir<R>(A.pnx[ii], A.pny[ii], nxn, nyn);
            const R txn = -nyn, tyn = nxn;
            const R s_x = A.sx[ii], s_y = A.sy[ii], q_x = A.qx[ii], q_y = A.qy[ii];
            const R sn = s_x * nxn + s_y * nyn;
            const R d2 = A.dscl[ii] * A.dscl[ii];
            if (sn > R(0)) {
                // slipping along the traction: counted as adhesion for this trial
                acc[1] += (double)(R(2) * d2 * (s_x * q_x + s_y * q_y));
                acc[2] += (double)(R(2) * d2 * (q_x * q_x + q_y * q_y));
                acc[0] += (double)(d2 * ((s_x + aj * q_x) * (s_x + aj * q_x) + (s_y + aj * q_y) * (s_y + aj * q_y)));
            } else {
                const R st = s_x * txn + s_y * tyn, rt = -st;
                const R qn = q_x * nxn + q_y * nyn, qt = q_x * txn + q_y * tyn;
                acc[1] -= (double)(R(2) * d2 * (rt * qt - rt * sn * dth_da));
                acc[2] -= (double)(R(2) * d2 * (-qt * qt + qt * sn * dth_da - rt * qn * dth_da));
                acc[3] -= (double)(R(2) * d2 * (qt * qn * dth_da));
                acc[0] += (double)(d2 * (st + aj * qt) * (st + aj * qt));
            }
        }
        block_sum<4>(red, acc);
        acc[0] += qa[0] + alpha_j * (2.0 * qa[1] + alpha_j * qa[2]);
        acc[1] += 2.0 * qa[1];
        acc[2] += 2.0 * qa[2];
        if (threadIdx.x == 0) {
            double *ta = S.tbl_alpha, *tr = S.tbl_rho, *td = S.tbl_drhoda;
            const double rhonew = acc[0];
            const double drho_da = acc[1] + alpha_j * acc[2] + alpha_j * alpha_j * acc[3];
            int itb = 1;
            while (itb <= j && alpha_j > ta[itb]) itb++;
            itb_u = itb;
            for (int k = j; k >= itb; k--) { ta[k + 1] = ta[k]; tr[k + 1] = tr[k]; td[k + 1] = td[k]; }
            if (has_bracket) {
                if (itb_a >= itb_u) itb_a++;
                if (itb_b >= itb_u) itb_b++;
                if (itb_x >= itb_u) itb_x++;
                if (itb_w >= itb_u) itb_w++;
                if (itb_v >= itb_u) itb_v++;
            }
            j++;
            ta[itb] = alpha_j; tr[itb] = rhonew; td[itb] = drho_da;
            bool prev_bracket = has_bracket;
            has_bracket = false;
            int ibrack = 1;
            while (ibrack < j - 1 && !has_bracket) {
                has_bracket = (tr[ibrack + 1] <= fmin(tr[ibrack], tr[ibrack + 2]));
                if (!has_bracket) ibrack++;
            }
            if (has_bracket && !prev_bracket) {
                itb_a = ibrack; itb_x = ibrack + 1; itb_b = ibrack + 2;
                if (tr[itb_a] < tr[itb_b]) { itb_w = itb_a; itb_v = itb_b; }
                else { itb_w = itb_b; itb_v = itb_a; }
                dst_prv1 = ta[itb_x] - ta[itb_w];
                dst_prv2 = ta[itb_w] - ta[itb_v];
            } else if (has_bracket) {
                if (tr[itb_u] <= tr[itb_x]) {
                    if (ta[itb_u] >= ta[itb_x]) itb_a = itb_x; else itb_b = itb_x;
                    itb_v = itb_w; itb_w = itb_x; itb_x = itb_u;
                } else {
                    if (ta[itb_u] < ta[itb_x]) itb_a = itb_u; else itb_b = itb_u;
                    if (tr[itb_u] <= tr[itb_w] || ta[itb_w] == ta[itb_x]) { itb_v = itb_w; itb_w = itb_u; }
                    else if (tr[itb_u] <= tr[itb_v] || ta[itb_v] == ta[itb_x] || ta[itb_v] == ta[itb_w]) itb_v = itb_u;
                }
                dst_prv2 = dst_prv1;
                dst_prv1 = dst_cur;
            }
            alpha_prv = alpha_j;
            double anew = alpha_j;
            if (has_bracket) {
                double xmid = 0.5 * (ta[itb_a] + ta[itb_b]);
                double tolx = eps_j * fabs(ta[itb_x]) + tiny;
                bool ldone = (fabs(ta[itb_x] - xmid) <= 2.0 * tolx - 0.5 * (ta[itb_b] - ta[itb_a]));
                if (!ldone) {
                    bool use_parab;
                    if (fabs(dst_prv2) <= tolx) use_parab = false;
                    else {
                        double br = (ta[itb_x] - ta[itb_w]) * (tr[itb_x] - tr[itb_v]);
                        double bq = (ta[itb_x] - ta[itb_v]) * (tr[itb_x] - tr[itb_w]);
                        double bp = (ta[itb_x] - ta[itb_v]) * bq - (ta[itb_x] - ta[itb_w]) * br;
                        bq = 2.0 * (bq - br);
                        if (bq > 0.0) bp = -bp;
                        bq = fabs(bq);
                        if (fabs(bp) >= fabs(0.5 * bq * dst_prv2) || bp <= bq * (ta[itb_a] - ta[itb_x]) ||
                            bp >= bq * (ta[itb_b] - ta[itb_x])) {
                            use_parab = false;
                        } else {
                            use_parab = true;
                            dst_cur = bp / bq;
                            double at = ta[itb_x] + dst_cur;
                            if (at - ta[itb_a] < 2.0 * tolx || ta[itb_b] - at < 2.0 * tolx)
                                dst_cur = tolx * dsign(1.0, xmid - ta[itb_x]);
                        }
                    }
                    if (!use_parab) {
                        if (ta[itb_x] >= xmid) dst_prv1 = ta[itb_a] - ta[itb_x];
                        else dst_prv1 = ta[itb_b] - ta[itb_x];
                        dst_cur = 0.381966 * dst_prv1;
                    }
                    anew = ta[itb_x] + dst_cur;
                }
            } else if (j == 1) {
                anew = alpha_j + 0.6 * alpha0;
                ddrho = 10.0;
            } else if (tr[j] < tr[1]) {
                int ib = j - 1;
                double dal = ta[ib + 1] - ta[ib];
                if (j < 3) { ddrho = (td[ib + 1] - td[ib]) / dal; anew = ta[ib + 1] + fmin(3.0 * dal, -td[ib] / ddrho); }
                else anew = ta[ib + 1] + 3.0 * dal;
            } else {
                int ib = 1;
                double dal = ta[ib + 1] - ta[ib];
                if (j < 3) { ddrho = (td[ib + 1] - td[ib]) / dal; anew = ta[ib] + fmin(-3.0 * dal, td[ib] / ddrho); }
                else anew = ta[ib] - 3.0 * dal;
            }
            bool stop = (j >= kMaxLs || fabs(anew - alpha_prv) < eps_j * fmax(fabs(anew), fabs(alpha_prv)));
            if (stop) {
                if (!has_bracket) S.nobracket = 1;
                if (j >= kMaxLs) {
                    int best = 1;
                    for (int k = 2; k <= kMaxLs; k++) if (tr[k] < tr[best]) best = k;
                    anew = ta[best];
                }
            }
            S.alpha_j = anew;
            S.stop_j = stop ? 1 : 0;
            S.jcount = j;
        }
        gsync();
        if (S.stop_j) break;
    }
    alpha_out = S.alpha_j;
    jout = S.jcount;
    bool ok = !S.nobracket;
    gsync();
    PHASE_END(P, O_T_LS - O_T_TOTAL, tls);
    return ok;
}

// slip s = A dp + ws on the interior (zero elsewhere)
template <typename T>
__device__ __noinline__ void compute_slip(const PView &P, const Ops<T> &op, int &nconv) {
    const int n = P.n;
    int *igs = P.igs();
    double *sx = P.c(W_SX), *sy = P.c(W_SY);
    const double *wsx = P.c(W_WSX), *wsy = P.c(W_WSY);
    FOR_I(i, n) { sx[i] = 0.0; sy[i] = 0.0; }
    prod_t<T>(op, P.c(W_DPX), P.c(W_DPY), sx, sy, OUT_INT, igs); nconv++;
    FOR_I(i, n) if (igs[i] >= Adhes) { sx[i] += wsx[i]; sy[i] += wsy[i]; }
    gsync();
}

// Mixed precision slip s = ws + A dp, with A dp = A dp_b + A (dp - dp_b): the base product
// A dp_b is an FP64 convolution, the change since the base an FP32 one.  The base is moved
// to the current dp (and re-evaluated in FP64) when the change exceeds tau * |dp| (rms over
// the grid); the FP32 part then carries at most ~tau times the FP32 rounding of the product.
constexpr double kRefreshTau = 5e-3;

__device__ __noinline__ void compute_slip_rr(const PView &P, const Ops<double> &op, const Ops<float> &o32,
                                             bool &have_base, int &nconv64, int &nconv32) {
    const int n = P.n;
    const int *igs = P.igs();
    const double *dpx = P.c(W_DPX), *dpy = P.c(W_DPY);
    double *dbx = P.c(W_DBX), *dby = P.c(W_DBY), *sbx = P.c(W_SBX), *sby = P.c(W_SBY);
    double *tx = P.c(W_TX), *ty = P.c(W_TY);
    double *sx = P.c(W_SX), *sy = P.c(W_SY);
    const double *wsx = P.c(W_WSX), *wsy = P.c(W_WSY);
    bool refresh = !have_base;
    if (have_base) {
        double a[2] = {0.0, 0.0};
        FOR_I(i, n) {
            const double ex = dpx[i] - dbx[i], ey = dpy[i] - dby[i];
            tx[i] = ex; ty[i] = ey;
            a[0] += ex * ex + ey * ey;
            a[1] += dpx[i] * dpx[i] + dpy[i] * dpy[i];
        }
        block_sum<2>(P.sm->red, a);
        refresh = a[0] > kRefreshTau * kRefreshTau * a[1];
    }
    if (refresh) {
        FOR_I(i, n) { dbx[i] = dpx[i]; dby[i] = dpy[i]; }
        prod_t<double>(op, dbx, dby, sbx, sby, OUT_ALL, igs); nconv64++;
        FOR_I(i, n) {
            if (igs[i] >= Adhes) { sx[i] = sbx[i] + wsx[i]; sy[i] = sby[i] + wsy[i]; }
            else { sx[i] = 0.0; sy[i] = 0.0; }
        }
        have_base = true;
        gsync();
        return;
    }
    FOR_I(i, n) {
        if (igs[i] >= Adhes) { sx[i] = sbx[i] + wsx[i]; sy[i] = sby[i] + wsy[i]; }
        else { sx[i] = 0.0; sy[i] = 0.0; }
    }
    prod_t<float>(o32, tx, ty, sx, sy, OUT_ADDINT, igs); nconv32++;
    gsync();
}

__device__ __noinline__ void set_nt(const PView &P) {
    const double *px = P.c(W_PX), *py = P.c(W_PY);
    double *nx = P.c(W_NX), *ny = P.c(W_NY);
    FOR_I(i, P.n) unit_dir(px[i], py[i], nx[i], ny[i]);
    gsync();
}

// ------------------------------------------------------------------------------------------
// GDsteady state in a storage precision S: the FP64 work columns, or FP32 columns for the
// single-precision part of mixed tier 4
// ------------------------------------------------------------------------------------------
template <typename S>
struct GdCols {
    S *px, *py, *pn, *dpx, *dpy, *trc, *dscl, *rx, *ry, *dvx, *dvy, *vx, *vy, *qx, *qy;
    S *pox, *poy, *sx, *sy, *nx, *ny, *zx, *zy, *wsx, *wsy, *pnx, *pny;
};
constexpr int kGdCols = 27;

template <typename S>
__device__ inline void gd_cols_assign(GdCols<S> &C, S *const (&a)[kGdCols]) {
    S **f[kGdCols] = {&C.px, &C.py, &C.pn, &C.dpx, &C.dpy, &C.trc, &C.dscl, &C.rx, &C.ry, &C.dvx, &C.dvy, &C.vx,
                      &C.vy, &C.qx, &C.qy, &C.pox, &C.poy, &C.sx, &C.sy, &C.nx, &C.ny, &C.zx, &C.zy, &C.wsx,
                      &C.wsy, &C.pnx, &C.pny};
    for (int k = 0; k < kGdCols; k++) *f[k] = a[k];
}

__device__ inline GdCols<double> gd_cols64(const PView &P) {
    double *const a[kGdCols] = {P.c(W_PX), P.c(W_PY), P.c(W_PN), P.c(W_DPX), P.c(W_DPY), P.c(W_TRC), P.c(W_DSCL),
                                P.c(W_RX), P.c(W_RY), P.c(W_DVX), P.c(W_DVY), P.c(W_VX), P.c(W_VY), P.c(W_QX),
                                P.c(W_QY), P.c(W_POX), P.c(W_POY), P.c(W_SX), P.c(W_SY), P.c(W_NX), P.c(W_NY),
                                P.c(W_ZX), P.c(W_ZY), P.c(W_WSX), P.c(W_WSY), P.c(W_PNX), P.c(W_PNY)};
    GdCols<double> C;
    gd_cols_assign(C, a);
    return C;
}

// FP32 state: 27 float columns in the double columns W_FST .. W_FST + 13
__device__ inline GdCols<float> gd_cols32(const PView &P) {
    float *b = (float *)P.c(W_FST);
    const size_t n = P.n;
    float *const a[kGdCols] = {b, b + n, b + 2 * n, b + 3 * n, b + 4 * n, b + 5 * n, b + 6 * n, b + 7 * n, b + 8 * n,
                               b + 9 * n, b + 10 * n, b + 11 * n, b + 12 * n, b + 13 * n, b + 14 * n, b + 15 * n,
                               b + 16 * n, b + 17 * n, b + 18 * n, b + 19 * n, b + 20 * n, b + 21 * n, b + 22 * n,
                               b + 23 * n, b + 24 * n, b + 25 * n, b + 26 * n};
    GdCols<float> C;
    gd_cols_assign(C, a);
    return C;
}

template <typename S>
__device__ inline LsArrays<S> ls_from_cols(const GdCols<S> &C) {
    LsArrays<S> A;
    A.dpx = C.dpx; A.dpy = C.dpy; A.dvx = C.dvx; A.dvy = C.dvy; A.vx = C.vx; A.vy = C.vy; A.qx = C.qx; A.qy = C.qy;
    A.sx = C.sx; A.sy = C.sy; A.nox = C.nx; A.noy = C.ny; A.dscl = C.dscl; A.trc = C.trc;
    A.pdx = nullptr; A.pdy = nullptr; A.pnx = C.pnx; A.pny = C.pny;
    return A;
}

template <typename S>
__device__ __noinline__ void gd_set_nt(const PView &P, const GdCols<S> &C) {
    FOR_I(i, P.n) unit_dir<S>(C.px[i], C.py[i], C.nx[i], C.ny[i]);
    gsync();
}

// residual of the scaled gradient: -dscl s (adhesion), its tangential part (slip)
template <typename S>
__device__ __noinline__ void gd_set_residual(const PView &P, const GdCols<S> &C) {
    const int *igs = P.igs();
    FOR_I(i, P.n) {
        if (igs[i] == Adhes) { C.rx[i] = -C.sx[i] * C.dscl[i]; C.ry[i] = -C.sy[i] * C.dscl[i]; }
        else if (igs[i] == Slip) {
            const S tx = -C.ny[i], ty = C.nx[i];
            const S st = tx * C.sx[i] + ty * C.sy[i];
            C.rx[i] = -st * tx * C.dscl[i]; C.ry[i] = -st * ty * C.dscl[i];
        } else { C.rx[i] = S(0); C.ry[i] = S(0); }
    }
    gsync();
}

// project_searchdir, gdsteady.f90:639-803 (variants E_trl, E_down(k), E_keep(f))
template <typename S>
__device__ __noinline__ void gd_project_searchdir(const PView &P, const GdCols<S> &C, int imeth, int kdown) {
    const PatchDesc &d = *P.d;
    const int mx = P.mx, my = P.my;
    const int *igs = P.igs();
    S *dvx = C.dvx, *dvy = C.dvy, *vx = C.vx, *vy = C.vy;
    const S *nx = C.nx, *ny = C.ny, *trc = C.trc;
    S *dxi = C.zx, *dyi = C.zy;   // copies of the input search direction (E_down)
    const S fac_v = S(1000), fdecay = (S)d.fdecay, zero = S(0);
    auto clampv = [&](S vt, S tb) { return (vt >= zero ? S(1) : S(-1)) * fmin(fabs(vt), fac_v * tb); };
    gsync();
    if (imeth == 2) { FOR_I(i, P.n) { dxi[i] = dvx[i]; dyi[i] = dvy[i]; } gsync(); }
    constexpr int U = ScanBatch<S>::U;
    FOR_ROW(iy, my) {
        const int i0 = iy * mx;
        int ii = (mx - 1) + i0;
        vx[ii] = zero; vy[ii] = zero;
        if (imeth != 2) {
            // E_trl (1) and E_keep (3): batched loads, the previous v carried in registers
            S vxn = zero, vyn = zero;
            for (int ixb = mx - 2; ixb >= 0; ixb -= U) {
                int el[U];
                S ex[U], ey[U], tx[U], ty[U], tb[U];
#pragma unroll
                for (int u = 0; u < U; u++) {
                    const int jj = ixb - u + i0;
                    el[u] = Exter; ex[u] = ey[u] = tx[u] = ty[u] = tb[u] = zero;
                    if (ixb - u >= 0) {
                        el[u] = igs[jj]; ex[u] = dvx[jj]; ey[u] = dvy[jj];
                        tx[u] = -ny[jj]; ty[u] = nx[jj]; tb[u] = trc[jj];
                    }
                }
#pragma unroll
                for (int u = 0; u < U; u++) {
                    if (ixb - u < 0) break;
                    const int jj = ixb - u + i0;
                    S wx, wy;
                    if (el[u] == Adhes) {
                        if (imeth == 1) { wx = vxn + ex[u]; wy = vyn + ey[u]; }
                        else {
                            wx = fdecay * vxn + ex[u]; wy = fdecay * vyn + ey[u];
                            dvx[jj] = wx - vxn; dvy[jj] = wy - vyn;
                        }
                    } else if (el[u] == Slip) {
                        const S vt = clampv(tx[u] * ex[u] + ty[u] * ey[u], tb[u]);
                        wx = tx[u] * vt; wy = ty[u] * vt;
                        dvx[jj] = wx - vxn; dvy[jj] = wy - vyn;
                    } else {
                        wx = zero; wy = zero;
                        dvx[jj] = -vxn; dvy[jj] = -vyn;
                    }
                    vx[jj] = wx; vy[jj] = wy;
                    vxn = wx; vyn = wy;
                }
            }
            continue;
        }
        for (int ix = mx - 2; ix >= 0; ix--) {
            ii = ix + i0;
            const S tx = -ny[ii], ty = nx[ii];
            if (imeth == 1) {
                if (igs[ii] == Adhes) { vx[ii] = vx[ii + 1] + dvx[ii]; vy[ii] = vy[ii + 1] + dvy[ii]; }
                else if (igs[ii] == Slip) {
                    const S vt = clampv(tx * dvx[ii] + ty * dvy[ii], trc[ii]);
                    vx[ii] = tx * vt; vy[ii] = ty * vt;
                    dvx[ii] = vx[ii] - vx[ii + 1]; dvy[ii] = vy[ii] - vy[ii + 1];
                } else {
                    vx[ii] = zero; vy[ii] = zero;
                    dvx[ii] = -vx[ii + 1]; dvy[ii] = -vy[ii + 1];
                }
            } else if (imeth == 2) {
                if (igs[ii] == Adhes) {
                    if (ix + 1 + kdown <= mx) {
                        vx[ii] = vx[ii + 1] + dxi[ii] - dxi[ii + kdown];
                        vy[ii] = vy[ii + 1] + dyi[ii] - dyi[ii + kdown];
                    } else { vx[ii] = vx[ii + 1] + dxi[ii]; vy[ii] = vy[ii + 1] + dyi[ii]; }
                    dvx[ii] = vx[ii] - vx[ii + 1]; dvy[ii] = vy[ii] - vy[ii + 1];
                } else {
                    if (igs[ii] == Slip) {
                        const S vt = clampv(tx * dxi[ii] + ty * dyi[ii], trc[ii]);
                        vx[ii] = tx * vt; vy[ii] = ty * vt;
                        dvx[ii] = vx[ii] - vx[ii + 1]; dvy[ii] = vy[ii] - vy[ii + 1];
                    } else {
                        vx[ii] = zero; vy[ii] = zero;
                        dvx[ii] = -vx[ii + 1]; dvy[ii] = -vy[ii + 1];
                    }
                    for (int kk = 1; kk <= kdown; kk++) if (ix + 1 + kk <= mx) { dxi[ii + kk] = zero; dyi[ii + kk] = zero; }
                }
            } else {
                if (igs[ii] == Adhes) {
                    vx[ii] = fdecay * vx[ii + 1] + dvx[ii]; vy[ii] = fdecay * vy[ii + 1] + dvy[ii];
                    dvx[ii] = vx[ii] - vx[ii + 1]; dvy[ii] = vy[ii] - vy[ii + 1];
                } else if (igs[ii] == Slip) {
                    const S vt = clampv(tx * dvx[ii] + ty * dvy[ii], trc[ii]);
                    vx[ii] = tx * vt; vy[ii] = ty * vt;
                    dvx[ii] = vx[ii] - vx[ii + 1]; dvy[ii] = vy[ii] - vy[ii + 1];
                } else {
                    vx[ii] = zero; vy[ii] = zero;
                    dvx[ii] = -vx[ii + 1]; dvy[ii] = -vy[ii + 1];
                }
            }
        }
    }
    gsync();
}

// compute_diagscaling on state S with element arithmetic in R.  R = float (mixed precision):
// the scaling is a preconditioner of the search direction, so single precision changes the
// iteration path only at rounding level of the direction
// for every element, the 1-based column of the last element at or behind it in its row that
// is not in adhesion (1 when there is none): one pass per row in place of a backward search
// per element
__device__ inline void trailing_nonadh(const PView &P, int *jxc) {
    const int mx = P.mx, my = P.my;
    const int *igs = P.igs();
    FOR_ROW(iy, my) {
        const int i0 = iy * mx;
        int last = 1;
        for (int ix = 1; ix <= mx; ix++) {
            if (igs[i0 + ix - 1] != Adhes) last = ix;
            jxc[i0 + ix - 1] = last;
        }
    }
    gsync();
}

template <typename S, typename R>
__device__ __noinline__ void gd_diagscaling(const PView &P, const GdCols<S> &C, const double coefs_d[2][2]) {
    const PatchDesc &d = *P.d;
    gsync();
    PHASE_START(tdg);
    const int mx = P.mx, n = P.n;
    const int *igs = P.igs();
    S *dscl = C.dscl;
    int *jxc = P.ci(I_JX);
    trailing_nonadh(P, jxc);
    R coefs[2][2] = {{(R)coefs_d[0][0], (R)coefs_d[0][1]}, {(R)coefs_d[1][0], (R)coefs_d[1][1]}};
    const R d_slp = (R)d.d_slp, pow_s = (R)d.pow_s;
    int ndeg = 0;
    FOR_I(ii, n) {
        const int el = igs[ii];
        if (el == Slip) {
            int elnew = Slip;
            R fac_s = R(0);
            if (!slip_element<R>(d, coefs, (R)C.px[ii], (R)C.py[ii], (R)C.pn[ii], (R)C.sx[ii], (R)C.sy[ii], elnew, fac_s)) ndeg++;
            else if (elnew == Slip) dscl[ii] = (S)(d_slp * pow_scaling<R>(fac_s, pow_s));
            else dscl[ii] = (S)dscl_adhesion<R>(d, ii % mx + 1, jxc[ii], (R)dscl[ii]);
        } else if (el == Adhes) {
            dscl[ii] = (S)dscl_adhesion<R>(d, ii % mx + 1, jxc[ii], (R)dscl[ii]);
        } else {
            dscl[ii] = S(0);
        }
    }
    ndeg = block_sumi1(P.sm->red, ndeg);
    if (ndeg > 0 && glead()) {
        // serial pass with the reference's carry-over of elnew and fac_s (elements in order)
        int elnew = Exter;
        R fac_s = R(0);
        for (int ii = 0; ii < n; ii++) {
            const int el = igs[ii];
            if (el == Slip) {
                int e2 = el;
                R f2 = fac_s;
                if (slip_element<R>(d, coefs, (R)C.px[ii], (R)C.py[ii], (R)C.pn[ii], (R)C.sx[ii], (R)C.sy[ii], e2, f2)) {
                    elnew = e2; fac_s = f2;
                }
            }
            if (el == Slip && elnew == Slip) dscl[ii] = (S)(d_slp * pow_scaling<R>(fac_s, pow_s));
            else if (el == Adhes || elnew == Adhes) dscl[ii] = (S)dscl_adhesion<R>(d, ii % mx + 1, jxc[ii], (R)dscl[ii]);
            else dscl[ii] = S(0);
        }
    }
    gsync();
    PHASE_END(P, O_T_DIAG - O_T_TOTAL, tdg);
}

// scalar state of the iteration, carried across the switch from FP32 to FP64 state
struct GdScal {
    int itgd, it_fb;
    double dif, difid, dif1, beta, alpha, alpha0;
    bool lchanged;
};

struct GdCtx {
    const Ops<double> *op64;
    const Ops<float> *o32;
    double coefs[2][2];
    double facnel;
    int tier;              // 0 plain, 1..4 mixed-precision tiers
    bool have_base;        // residual replacement base valid (FP64 state)
    int nconv64, nconv32, nls;
};

// slip s = ws + A dp: FP64 product, FP64 base + FP32 change (mixed, FP64 state), or FP32
template <typename S>
__device__ __noinline__ void gd_slip(const PView &P, const GdCols<S> &C, GdCtx &X) {
    if constexpr (sizeof(S) == 8) {
        if (X.o32) compute_slip_rr(P, *X.op64, *X.o32, X.have_base, X.nconv64, X.nconv32);
        else compute_slip<double>(P, *X.op64, X.nconv64);
    } else {
        const int n = P.n;
        const int *igs = P.igs();
        FOR_I(i, n) { C.sx[i] = 0.0f; C.sy[i] = 0.0f; }
        prod_t<float, float>(*X.o32, C.dpx, C.dpy, C.sx, C.sy, OUT_INT, igs); X.nconv32++;
        FOR_I(i, n) if (igs[i] >= Adhes) { C.sx[i] += C.wsx[i]; C.sy[i] += C.wsy[i]; }
        gsync();
    }
}

// search-direction product q = A dv
template <typename S>
__device__ inline void gd_product_q(const PView &P, const GdCols<S> &C, GdCtx &X) {
    const int *igs = P.igs();
    if constexpr (sizeof(S) == 8) {
        if (X.o32) { prod_t<float, double>(*X.o32, C.dvx, C.dvy, C.qx, C.qy, OUT_INT, igs); X.nconv32++; }
        else { prod_t<double, double>(*X.op64, C.dvx, C.dvy, C.qx, C.qy, OUT_INT, igs); X.nconv64++; }
    } else {
        prod_t<float, float>(*X.o32, C.dvx, C.dvy, C.qx, C.qy, OUT_INT, igs); X.nconv32++;
    }
}

template <typename S>
__device__ inline bool gd_linesearch(const PView &P, const GdCols<S> &C, GdCtx &X, double alpha0, double &alpha, int &its) {
    if constexpr (sizeof(S) == 8) {
        if (X.o32 && X.tier == 3) {
            LsArrays<float> A;
            ls_arrays(P, A);
            return perform_linesearch<float>(P, A, alpha0, alpha, its);
        }
    }
    return perform_linesearch<S>(P, ls_from_cols<S>(C), alpha0, alpha, its);
}

template <typename S>
__device__ inline void gd_scaling(const PView &P, const GdCols<S> &C, const GdCtx &X) {
    if constexpr (sizeof(S) == 8) {
        if (X.o32 && X.tier >= 2) gd_diagscaling<double, float>(P, C, X.coefs);
        else gd_diagscaling<double, double>(P, C, X.coefs);
    } else {
        gd_diagscaling<float, float>(P, C, X.coefs);
    }
}

// dif (change of p, scaled by facdif) and difid (tolerance eps_stop) after an iteration
template <typename S>
__device__ inline void gd_difs(const PView &P, const GdCols<S> &C, const GdCtx &X, GdScal &g, double eps_stop,
                               bool with_change) {
    const int n = P.n;
    double facdif;
    if (g.beta >= 0.1) facdif = 1.0;
    else if (g.beta >= 0.001) facdif = 0.1 / g.beta;
    else facdif = 100.0;
    double a[2] = {0, 0};
    FOR_I(i, n) {
        if (with_change) {
            const S ex = C.pox[i] - C.px[i], ey = C.poy[i] - C.py[i];
            a[0] += (double)(ex * ex + ey * ey);
        }
        a[1] += (double)(C.px[i] * C.px[i] + C.py[i] * C.py[i]);
    }
    block_sum<2>(P.sm->red, a);
    if (with_change) g.dif = X.facnel * sqrt(a[0] / (2 * n)) * facdif;
    g.difid = eps_stop * fmax(1e-6, X.facnel * sqrt(a[1] / (2 * n)));
}

// the GDsteady iterations (gdsteady.f90:9-606) on state S until the stopping test with
// tolerance eps_stop holds or maxgd is reached; false on a failed line search
template <typename S>
__device__ __noinline__ bool gd_iterate(const PView &P, const GdCols<S> &C, GdCtx &X, GdScal &g, double eps_stop,
                                        int maxgd) {
    const PatchDesc &d = *P.d;
    const int n = P.n;
    RedSmem &red = P.sm->red;
    int *igs = P.igs(), *igsold = P.ci(I_OLD);
    const S tiny = S(1e-12);
    const bool r32 = (sizeof(S) == 4) || (X.o32 && X.tier >= 2);
    while ((g.lchanged || g.dif > g.difid) && g.itgd < maxgd) {
        g.itgd++;
        FOR_I(i, n) { C.dvx[i] = C.rx[i]; C.dvy[i] = C.ry[i]; }
        int imeth, kdown;
        if (g.beta > d.betath || g.itgd - g.it_fb <= 1) { imeth = d.gd_meth; kdown = d.kdown; }
        else { imeth = 2; kdown = d.kdowfb; g.it_fb = g.itgd; }
        gd_project_searchdir<S>(P, C, imeth, kdown);
        gd_product_q<S>(P, C, X);
        if (g.itgd <= 1) {
            double a[2] = {0, 0};
            FOR_I(i, n) {
                a[0] += (double)(C.rx[i] * C.rx[i] + C.ry[i] * C.ry[i]);
                a[1] += (double)((C.rx[i] * C.qx[i] + C.ry[i] * C.qy[i]) * C.dscl[i]);
            }
            block_sum<2>(red, a);
            g.alpha0 = a[0] / a[1];
        } else {
            g.alpha0 = 0.5 * (g.alpha0 + g.alpha);
        }
        int its_j = 0;
        if (!gd_linesearch<S>(P, C, X, g.alpha0, g.alpha, its_j)) return false;
        X.nls += its_j;
        {
            double a[2] = {0, 0};
            FOR_I(i, n) if (igs[i] >= Adhes) {
                const S a0 = C.dscl[i] * C.qx[i], a1 = C.dscl[i] * C.qy[i];
                a[0] += (double)(a0 * a0 + a1 * a1);
                a[1] += (double)(C.rx[i] * C.rx[i] + C.ry[i] * C.ry[i]);
            }
            block_sum<2>(red, a);
            g.beta = g.alpha * sqrt(a[0]) / sqrt(a[1]);
        }
        const S al = (S)g.alpha;
        FOR_I(i, n) {
            igsold[i] = igs[i];
            C.pox[i] = C.px[i]; C.poy[i] = C.py[i];
            if (igs[i] >= Adhes) { C.dpx[i] += al * C.dvx[i]; C.dpy[i] += al * C.dvy[i]; }
        }
        apply_trcbnd<S>(P, C.trc, C.dpx, C.dpy, C.px, C.py);
        gd_set_nt<S>(P, C);
        gd_slip<S>(P, C, X);
        // local optimisation (solve_elmtrc) and active-set updates
        int chg = 0;
        FOR_I(ii, n) {
            if (igsold[ii] == Slip) {
                int elnew = igs[ii];
                double cosdth;
                if (r32) {
                    // single precision: the local element solve only feeds the release test below
                    float prf[3] = {(float)C.px[ii], (float)C.py[ii], (float)C.pn[ii]};
                    float sif[2] = {(float)C.sx[ii], (float)C.sy[ii]};
                    const float cf[2][2] = {{(float)X.coefs[0][0], (float)X.coefs[0][1]},
                                            {(float)X.coefs[1][0], (float)X.coefs[1][1]}};
                    elm_solve<float>(elnew, cf, 1e-6f, 1.0f, 1.0f, prf, (float)d.fstat, sif);
                    cosdth = (double)(((float)C.nx[ii] * prf[0] + (float)C.ny[ii] * prf[1]) / (float)C.trc[ii]);
                } else {
                    double pr[3] = {(double)C.px[ii], (double)C.py[ii], (double)C.pn[ii]};
                    double si[2] = {(double)C.sx[ii], (double)C.sy[ii]};
                    elm_solve<double>(elnew, X.coefs, 1e-6, 1.0, 1.0, pr, d.fstat, si);
                    cosdth = ((double)C.nx[ii] * pr[0] + (double)C.ny[ii] * pr[1]) / (double)C.trc[ii];
                }
                const S snrm = C.nx[ii] * C.sx[ii] + C.ny[ii] * C.sy[ii];
                // the A->S test below only sees elements that were in adhesion
                if ((snrm > S(0) && (C.dscl[ii] >= S(0.001) || elnew == Adhes)) || cosdth <= -0.5) { igs[ii] = Adhes; chg = 1; }
            } else if (igs[ii] == Adhes) {
                const S ptabs = sqrt(C.px[ii] * C.px[ii] + C.py[ii] * C.py[ii]);
                if (ptabs >= C.trc[ii] - tiny) { igs[ii] = Slip; chg = 1; }
            }
        }
        chg = block_sumi1(red, chg);
        g.lchanged = chg > 0;
        gd_scaling<S>(P, C, X);
        gd_set_residual<S>(P, C);
        gd_difs<S>(P, C, X, g, eps_stop, true);
        if (g.itgd == 1) g.dif1 = g.dif;
    }
    return true;
}

// set-up of the iteration on state S: traction bound, dp, normals, slip, scaling, residual
template <typename S>
__device__ __noinline__ void gd_start(const PView &P, const GdCols<S> &C, GdCtx &X, GdScal &g, bool fresh) {
    const PatchDesc &d = *P.d;
    const int n = P.n, mx = P.mx;
    const S fstat = (S)d.fstat;
    FOR_I(i, n) {
        C.trc[i] = fstat * C.pn[i];
        if (fresh) C.dscl[i] = S(1);
    }
    if (fresh) {
        FOR_I(ii, n) {
            const int ix = ii % mx;
            if (ix == mx - 1) { C.dpx[ii] = C.px[ii]; C.dpy[ii] = C.py[ii]; }
            else { C.dpx[ii] = C.px[ii] - C.px[ii + 1]; C.dpy[ii] = C.py[ii] - C.py[ii + 1]; }
        }
    }
    gsync();
    gd_set_nt<S>(P, C);
    gd_slip<S>(P, C, X);
    gd_scaling<S>(P, C, X);
    gd_set_residual<S>(P, C);
    if (fresh) {
        double m = 0.0;
        FOR_I(i, n) m = fmax(m, fmax(fabs((double)C.rx[i]), fabs((double)C.ry[i])));
        m = block_max1(P.sm->red, m);
        if (m < 1e-12) g.dif = 0.0;
    }
}

// switch tolerance of tier 4: the FP32 iteration stops where single precision stops
// resolving the change of the tractions; the FP64 iteration continues from there
constexpr double kGdSwitchEps = 1e-5;

// gdsteady, gdsteady.f90:9-606 (elastic).  Returns itgd (negated on stagnation);
// lstagn as in the reference; returns -100000 when the line search has no bracket.
// Mixed precision (o32 != nullptr): tiers 1-3 run the FP64 iteration with FP32 products
// (see compute_slip_rr) and, from tier 2, FP32 element arithmetic; tier 4 runs the same
// iteration on an FP32 state until its change falls below kGdSwitchEps and then continues
// it, without a restart, on the FP64 state with tier-2 arithmetic.
template <typename T>
__device__ __noinline__ int gdsteady(const PView &P, const Ops<T> &op, int maxgd, double eps, double &err, bool &lstagn,
                        int &nconv, int &nls, const Ops<float> *o32, int &nconv32) {
    const PatchDesc &d = *P.d;
    const int n = P.n, mx = P.mx, my = P.my;
    RedSmem &red = P.sm->red;
    const int *igs = P.igs();
    GdCtx X;
    X.op64 = &op; X.o32 = o32; X.tier = o32 ? d.precision : 0; X.have_base = false;
    X.nconv64 = 0; X.nconv32 = 0; X.nls = 0;
    const size_t bsz = (size_t)4 * mx * my;
    const size_t o0 = (size_t)mx + (size_t)my * 2 * mx;
    X.coefs[0][0] = d.cf[0 * bsz + o0] / d.ga;
    X.coefs[0][1] = d.cf[1 * bsz + o0] / d.ga;
    X.coefs[1][0] = X.coefs[0][1];
    X.coefs[1][1] = d.cf[2 * bsz + o0] / d.ga;
    int nadh, nslip, nplast, nexter;
    count_eldiv(P, nadh, nslip, nplast, nexter);
    X.facnel = sqrt((double)(float)n / (double)(float)(nadh + nslip + nplast));
    GdScal g;
    g.itgd = 0; g.it_fb = -99; g.dif = 2.0; g.difid = 1.0; g.dif1 = 0.0; g.beta = 1.0; g.alpha = 0.0; g.alpha0 = 0.0;
    g.lchanged = false;
    lstagn = false;
    const GdCols<double> C64 = gd_cols64(P);
    bool ok = true;
    if (o32 && X.tier >= 4) {
        const GdCols<float> C32 = gd_cols32(P);
        FOR_I(i, n) {
            C32.pn[i] = (float)C64.pn[i]; C32.px[i] = (float)C64.px[i]; C32.py[i] = (float)C64.py[i];
            C32.wsx[i] = (float)C64.wsx[i]; C32.wsy[i] = (float)C64.wsy[i];
        }
        gsync();
        gd_start<float>(P, C32, X, g, true);
        ok = gd_iterate<float>(P, C32, X, g, fmax(eps, kGdSwitchEps), maxgd);
        // continue on the FP64 state: same iteration counters, step lengths and scaling
        FOR_I(i, n) {
            C64.px[i] = C32.px[i]; C64.py[i] = C32.py[i]; C64.dpx[i] = C32.dpx[i]; C64.dpy[i] = C32.dpy[i];
            C64.dscl[i] = C32.dscl[i];
        }
        gsync();
        X.tier = 2;
        if (ok) {
            gd_start<double>(P, C64, X, g, false);
            gd_difs<double>(P, C64, X, g, eps, false);
        }
    } else {
        gd_start<double>(P, C64, X, g, true);
    }
    if (ok) ok = gd_iterate<double>(P, C64, X, g, eps, maxgd);
    nconv += X.nconv64; nconv32 += X.nconv32; nls += X.nls;
    if (!ok) { err = g.dif; return -100000; }
    double resrms;
    {
        double a = 0; int c = 0;
        FOR_I(i, n) if (igs[i] >= Adhes) { a += C64.rx[i] * C64.rx[i] + C64.ry[i] * C64.ry[i]; c += 2; }
        a = block_sum1(red, a); c = block_sumi1(red, c);
        resrms = sqrt(a / max(1, c));
    }
    const double tiny = 1e-12;
    double res_dp = resrms / fmax(X.coefs[0][0], X.coefs[1][1]);
    err = g.dif;
    double conv = 1.0;
    if (g.dif * g.dif1 > 0.0 && g.itgd > 1) conv = exp(log(g.dif / g.dif1) / (g.itgd - 1));
    int itgd = g.itgd;
    if (g.lchanged && itgd >= maxgd) lstagn = true;
    else if (g.dif > g.difid && conv > 1.0 && itgd >= maxgd) lstagn = true;
    else if (conv < 1.0 - tiny && res_dp > 5.0 * g.difid / (1.0 - conv)) { itgd = -itgd; lstagn = true; }
    return itgd;
}

// ------------------------------------------------------------------------------------------
// TangCG, m_solvpt.f90:1841-2442 (elastic).  The FFT preconditioner uses blocks xx, yy of
// the preconditioner spectra, evaluated at the convolution's FFT size.
// ------------------------------------------------------------------------------------------
// p0x, p0y (sensitivity solves, m_solvpt.f90:1908-1914): the tolerance is relative to the change
// of the tractions from p0 instead of to the tractions
template <typename T>
__device__ __noinline__ int tangcg(const PView &P, const Ops<T> &op, const T *Mxx, const T *Myy, int maxcg, double eps,
                      double &err, int &nconv, const double *p0x = nullptr, const double *p0y = nullptr) {
    const PatchDesc &d = *P.d;
    const int n = P.n, my = P.my, mx = P.mx;
    RedSmem &red = P.sm->red;
    int *igs = P.igs();
    double *px = P.c(W_PX), *py = P.c(W_PY), *pn = P.c(W_PN), *g = P.c(W_TRC);
    double *sx = P.c(W_SX), *sy = P.c(W_SY), *wsx = P.c(W_WSX), *wsy = P.c(W_WSY);
    double *nx = P.c(W_NX), *ny = P.c(W_NY), *rx = P.c(W_RX), *ry = P.c(W_RY);
    double *zx = P.c(W_ZX), *zy = P.c(W_ZY), *vx = P.c(W_VX), *vy = P.c(W_VY);
    double *qx = P.c(W_QX), *qy = P.c(W_QY), *pox = P.c(W_POX), *poy = P.c(W_POY);
    const size_t bsz = (size_t)4 * mx * my;
    const size_t o0 = (size_t)mx + (size_t)my * 2 * mx;
    const double cxx = d.cf[0 * bsz + o0], cyy = d.cf[2 * bsz + o0], ga = d.ga;
    const int num_inn = 4;
    const double small = 1e-6;
    bool use_fftprec = true;
    int nadh, nslip, nplast, nexter;
    count_eldiv(P, nadh, nslip, nplast, nexter);
    const double facnel = sqrt((double)(float)n / (double)(float)(nadh + nslip + nplast));
    FOR_I(i, n) g[i] = d.fstat * pn[i];
    int itcg = 0, it_inn = 0;
    double dif = 2.0, difid = 1.0, difinn = 0.0, alpha = 0.0, trsinn = 0.0;
    bool lchanged = false;
    set_nt(P);
    FOR_I(i, n) { sx[i] = 0.0; sy[i] = 0.0; }
    prod_t<T>(op, px, py, sx, sy, OUT_INT, igs); nconv++;
    auto set_r = [&]() {
        FOR_I(i, n) {
            double r0 = -sx[i], r1 = -sy[i];
            if (igs[i] == Slip) {
                const double tx = -ny[i], ty = nx[i];
                double perp = tx * r0 + ty * r1; r0 = perp * tx; r1 = perp * ty;
            }
            rx[i] = r0; ry[i] = r1;
        }
        gsync();
    };
    FOR_I(i, n) if (igs[i] >= Adhes) { sx[i] += wsx[i]; sy[i] += wsy[i]; }
    gsync();
    set_r();
    while ((lchanged || dif > difid) && itcg < maxcg) {
        itcg++; it_inn++;
        if (use_fftprec) {
            if (nslip + nplast > 3 * nadh && my > 1) use_fftprec = false;
            if (itcg >= maxcg / 2) use_fftprec = false;
            if (!use_fftprec) lchanged = true;
        }
        if (use_fftprec) {
            convolve<T, double>(op.cv, rx, nullptr, zx, nullptr, 1, Mxx, nullptr, nullptr, OUT_INT, igs);
            convolve<T, double>(op.cv, ry, nullptr, zy, nullptr, 1, Myy, nullptr, nullptr, OUT_INT, igs);
            nconv++;
        } else {
            FOR_I(i, n) { zx[i] = rx[i]; zy[i] = ry[i]; }
        }
        FOR_I(i, n) {
            double z0 = zx[i], z1 = zy[i];
            if (igs[i] == Slip) {
                double snrm = -sx[i] * nx[i] - sy[i] * ny[i];
                z0 = z0 / (cxx + ga * snrm / g[i]);
                z1 = z1 / (cyy + ga * snrm / g[i]);
                const double tx = -ny[i], ty = nx[i];
                double perp = tx * z0 + ty * z1; z0 = perp * tx; z1 = perp * ty;
            } else {
                z0 = z0 / cxx; z1 = z1 / cyy;
            }
            zx[i] = z0; zy[i] = z1;
        }
        gsync();
        if (itcg <= 1 || lchanged) {
            FOR_I(i, n) { vx[i] = zx[i]; vy[i] = zy[i]; }
        } else {
            double a[2] = {0, 0};
            FOR_I(i, n) { a[0] += zx[i] * qx[i] + zy[i] * qy[i]; a[1] += vx[i] * qx[i] + vy[i] * qy[i]; }
            block_sum<2>(red, a);
            double zq = a[0], vq = a[1], beta;
            if (fabs(zq) < 1e-60 || fabs(vq) < small * fabs(zq)) beta = 0.0;
            else beta = -zq / vq;
            FOR_I(i, n) { vx[i] = beta * vx[i] + zx[i]; vy[i] = beta * vy[i] + zy[i]; }
        }
        gsync();
        prod_t<T>(op, vx, vy, qx, qy, OUT_INT, igs); nconv++;
        FOR_I(i, n) if (igs[i] == Slip) {
            const double tx = -ny[i], ty = nx[i];
            double perp = tx * qx[i] + ty * qy[i];
            double q0 = perp * tx, q1 = perp * ty;
            double snrm = (nx[i] * sx[i] + ny[i] * sy[i]) / g[i];
            qx[i] = q0 - snrm * vx[i]; qy[i] = q1 - snrm * vy[i];
        }
        double rv, vq;
        {
            double a[2] = {0, 0};
            FOR_I(i, n) { a[0] += rx[i] * vx[i] + ry[i] * vy[i]; a[1] += vx[i] * qx[i] + vy[i] * qy[i]; }
            block_sum<2>(red, a);
            rv = a[0]; vq = a[1];
        }
        if (fabs(rv) < 1e-60) alpha = 0.0;
        else if (fabs(vq) < small * fabs(rv)) alpha = 1.0;
        else alpha = rv / vq;
        {
            double a[2] = {0, 0};
            FOR_I(i, n) {
                pox[i] = px[i]; poy[i] = py[i];
                if (igs[i] >= Adhes) { px[i] += alpha * vx[i]; py[i] += alpha * vy[i]; }
                if (igs[i] == Slip) {
                    double ptabs = sqrt(px[i] * px[i] + py[i] * py[i]);
                    px[i] = px[i] * g[i] / ptabs; py[i] = py[i] * g[i] / ptabs;
                }
                a[0] += vx[i] * vx[i] + vy[i] * vy[i];
                if (p0x) {
                    const double ex = px[i] - p0x[i], ey = py[i] - p0y[i];
                    a[1] += ex * ex + ey * ey;
                } else {
                    a[1] += px[i] * px[i] + py[i] * py[i];
                }
            }
            block_sum<2>(red, a);
            dif = alpha * facnel * sqrt(a[0] / (2 * n));
            difinn += dif;
            if (itcg <= 5 || itcg % 5 == 1) {
                double ptang = facnel * sqrt(a[1] / (2 * n));
                difid = eps * fmax(1e-6, ptang);
                trsinn = (double)0.01f * ptang;
            }
        }
        if (it_inn >= num_inn || dif <= difid || difinn > trsinn) {
            int chg = 0;
            FOR_I(i, n) if (igs[i] == Adhes) {
                double ptabs = sqrt(px[i] * px[i] + py[i] * py[i]);
                if (ptabs > g[i]) {
                    igs[i] = Slip; px[i] = px[i] * g[i] / ptabs; py[i] = py[i] * g[i] / ptabs; chg = 1;
                }
            }
            prod_t<T>(op, px, py, sx, sy, OUT_INT, igs); nconv++;
            FOR_I(i, n) if (igs[i] >= Adhes) { sx[i] += wsx[i]; sy[i] += wsy[i]; }
            FOR_I(i, n) if (igs[i] == Slip) {
                double snrm = sx[i] * px[i] + sy[i] * py[i];
                if (snrm > 0.0) { igs[i] = Adhes; chg = 1; }
            }
            chg = block_sumi1(red, chg);
            lchanged = chg > 0;
            double a = 0;
            FOR_I(i, n) { double ex = pox[i] - px[i], ey = poy[i] - py[i]; a += ex * ex + ey * ey; }
            a = block_sum1(red, a);
            dif = facnel * sqrt(a / (2 * n));
            it_inn = 0;
            difinn = 0.0;
            if (lchanged) count_eldiv(P, nadh, nslip, nplast, nexter);
        }
        if ((lchanged || dif > difid) && itcg < maxcg) {
            if (it_inn <= 0) { set_nt(P); set_r(); }
            else { FOR_I(i, n) if (igs[i] >= Adhes) { rx[i] -= alpha * qx[i]; ry[i] -= alpha * qy[i]; } gsync(); }
        }
    }
    err = dif;
    return itcg;
}

} // namespace cgb
