// CPU ORACLE -- test infrastructure only (see contact_oracle.h).
//
// Influence coefficients (Boussinesq-Cerruti, piecewise constant loading) and the
// products u = A p: FFT-based (fft_VecAijPj) and direct row sums (gf3_AijPj), plus
// the FFT preconditioner (fft_makePrec).
#pragma once
#include "orc_core.hpp"

namespace orc {

// elascf_pcwcns, m_visc.f90:431-604
inline void elascf_pcwcns(double akv, double nuv, int mx, int my, double dx, double dy,
                          double xshft, double yshft, Inflcf &cs) {
    const int W = 2 * mx + 1;                      // arrays (-mx:mx, -my:my)
    auto id = [&](int ix, int iy) { return (size_t)(ix + mx) + (size_t)(iy + my) * W; };
    std::vector<double> r((size_t)W * (2 * my + 1)), x(r.size()), y(r.size()), xly2y1(r.size()), ylx2x1(r.size());
    const double e1 = (1.0 - nuv) / pi, e2 = 1.0 / pi, e3 = nuv / pi;
    const double tolx = dx * 1e-10, tolx2 = dx * 1e-20;
    for (int ik = 1; ik <= 3; ik++) for (int jk = 1; jk <= 3; jk++)
        std::fill(cs.cf[ik - 1][jk - 1].begin(), cs.cf[ik - 1][jk - 1].end(), 0.0);
    int iy0 = -my;
    if (my == 1) iy0 = -my + 1;
    for (int iy = iy0; iy <= my; iy++)
        for (int ix = -mx; ix <= mx; ix++) {
            x[id(ix, iy)] = (double)(float)ix * dx + xshft - 0.5 * dx;
            y[id(ix, iy)] = (double)(float)iy * dy + yshft - 0.5 * dy;
            r[id(ix, iy)] = std::sqrt(x[id(ix, iy)] * x[id(ix, iy)] + y[id(ix, iy)] * y[id(ix, iy)]);
        }
    for (int iy = iy0; iy <= my - 1; iy++)
        for (int ix = -mx; ix <= mx - 1; ix++) {
            double &c = cs.at(ix, iy, 2, 1);
            c = c - e3 * r[id(ix, iy)];
            c = c + e3 * r[id(ix, iy + 1)];
            c = c + e3 * r[id(ix + 1, iy)];
            c = c - e3 * r[id(ix + 1, iy + 1)];
        }
    if (std::fabs(akv) >= 1e-6) {
        std::vector<double> alr(r.size()), atxy(r.size()), atyx(r.size());
        for (int iy = iy0; iy <= my; iy++)
            for (int ix = -mx; ix <= mx; ix++) {
                size_t k = id(ix, iy);
                alr[k] = std::log(r[k]);
                atyx[k] = std::atan(y[k] / (x[k] + tolx2));
                atxy[k] = std::atan(x[k] / (y[k] + tolx2));
            }
        for (int iy = iy0; iy <= my - 1; iy++)
            for (int ix = -mx; ix <= mx - 1; ix++) {
                auto j5 = [&](int a, int b) { size_t k = id(a, b); return y[k] * alr[k] + x[k] * atyx[k]; };
                auto j6 = [&](int a, int b) { size_t k = id(a, b); return x[k] * alr[k] + y[k] * atxy[k]; };
                double &c13 = cs.at(ix, iy, 1, 3);
                c13 = c13 - e2 * akv * j5(ix, iy);
                c13 = c13 + e2 * akv * j5(ix, iy + 1);
                c13 = c13 + e2 * akv * j5(ix + 1, iy);
                c13 = c13 - e2 * akv * j5(ix + 1, iy + 1);
                double &c23 = cs.at(ix, iy, 2, 3);
                c23 = c23 - e2 * akv * j6(ix, iy);
                c23 = c23 + e2 * akv * j6(ix, iy + 1);
                c23 = c23 + e2 * akv * j6(ix + 1, iy);
                c23 = c23 - e2 * akv * j6(ix + 1, iy + 1);
            }
    }
    for (int iy = iy0; iy <= my - 1; iy++)
        for (int ix = -mx; ix <= mx; ix++) {
            size_t a = id(ix, iy), b = id(ix, iy + 1);
            if (std::min(std::fabs(y[a] + r[a]), std::fabs(y[b] + r[b])) < tolx) xly2y1[a] = 0.0;
            else xly2y1[a] = x[a] * std::log((y[b] + r[b]) / (y[a] + r[a]));
        }
    for (int iy = iy0; iy <= my; iy++)
        for (int ix = -mx; ix <= mx - 1; ix++) {
            size_t a = id(ix, iy), b = id(ix + 1, iy);
            if (std::min(std::fabs(x[a] + r[a]), std::fabs(x[b] + r[b])) < tolx) ylx2x1[a] = 0.0;
            else ylx2x1[a] = y[a] * std::log((x[b] + r[b]) / (x[a] + r[a]));
        }
    for (int iy = iy0; iy <= my - 1; iy++)
        for (int ix = -mx; ix <= mx - 1; ix++) {
            double X0 = xly2y1[id(ix, iy)], X1 = xly2y1[id(ix + 1, iy)];
            double Y0 = ylx2x1[id(ix, iy)], Y1 = ylx2x1[id(ix, iy + 1)];
            double &c33 = cs.at(ix, iy, 3, 3);
            c33 = c33 - e1 * (X0 + Y0);
            c33 = c33 + e1 * (X1 + Y1);
            double &c11 = cs.at(ix, iy, 1, 1);
            c11 = c11 - (e1 * X0 + e2 * Y0);
            c11 = c11 + (e1 * X1 + e2 * Y1);
            double &c22 = cs.at(ix, iy, 2, 2);
            c22 = c22 - (e1 * Y0 + e2 * X0);
            c22 = c22 + (e1 * Y1 + e2 * X1);
        }
    for (int iy = iy0; iy <= my - 1; iy++)
        for (int ix = -mx; ix <= mx - 1; ix++) {
            cs.at(ix, iy, 3, 1) = -cs.at(ix, iy, 1, 3);
            cs.at(ix, iy, 3, 2) = -cs.at(ix, iy, 2, 3);
            cs.at(ix, iy, 1, 2) = cs.at(ix, iy, 2, 1);
        }
}

// gf3_AijPj, m_aijpj.f90:99-254: one row of A times p, restricted to the row extents of
// p's element division (pe).
inline double aijpj(int ii, int ik, const GF3 &p, const Eldiv &pe, int jkarg, const Inflcf &c, int mx, int my) {
    int jk0, jk1;
    if (jkarg == -3) {
        jk0 = 1; jk1 = 3;
        if (!c.nt_cpl && ik <= 2) jk1 = 2;
        if (!c.nt_cpl && ik == 3) jk0 = 3;
    } else if (jkarg == -2) {
        jk0 = 1; jk1 = 2;
        if (!c.nt_cpl && ik == 3) jk1 = 0;
    } else if (jkarg >= 1 && jkarg <= 3) {
        jk0 = jk1 = jkarg;
        if (!c.nt_cpl && ik <= 2) jk1 = std::min(2, jk1);
        if (!c.nt_cpl && ik == 3) jk0 = 3;
    } else { jk0 = 1; jk1 = 0; }
    int ix = ii % mx + 1, iy = ii / mx + 1;
    double partsum = 0.0;
    for (int jy = 1; jy <= my; jy++)
        for (int jk = jk0; jk <= jk1; jk++) {
            int jh2 = (jy - 1) * mx;
            double rowsum = 0.0;
            int j0 = std::max(1, pe.row1st[jy - 1] - 1), j1 = std::min(mx, pe.rowlst[jy - 1] + 1);
            const double *pv = p.col(jk);
            for (int jx = j0; jx <= j1; jx++)
                rowsum += c.at(ix - jx, iy - jy, ik, jk) * pv[(jx - 1) + jh2];
            partsum += rowsum;
        }
    partsum *= c.ga_inv;
    // the layer's own term (m_aijpj.f90:246-252); jkarg -2 and -3 both contain direction ik
    if (c.use_3bl && ik <= ikY && (jkarg == ik || jkarg <= ikTANG)) partsum += c.flx_3bl * p.col(ik)[ii];
    return partsum;
}

// fft_VecAijPj, m_aijpj.f90:712-1015: u_ik (+)= C_ik,jk * p_jk on the elements of igs in iigs.
// igs is the output element division, pe the one carried by p.
inline void fft_vecaijpj(const Eldiv &igs, bool ladd, int iigs, GF3 &u, int ik, const GF3 &p,
                         const Eldiv &pe, int jk, Inflcf &c, int mx, int my) {
    int ix0, ix1, iy0, iy1, iarea;
    if (iigs == AllInt) {
        ix0 = std::max(1, std::min(igs.ixmin - 1, pe.ixmin - 1));
        ix1 = std::min(mx, std::max(igs.ixmax + 1, pe.ixmax + 1));
        iy0 = std::min(igs.iymin, pe.iymin);
        iy1 = std::max(igs.iymax, pe.iymax);
        iarea = (ix1 - ix0 + 1) * (iy1 - iy0 + 1);
    } else {
        iarea = 0;
    }
    if (iigs != AllInt || 1.1f * (float)iarea > (float)(mx * my)) {
        ix0 = 1; ix1 = mx; iy0 = 1; iy1 = my;
    }
    int g0, g1; igsrange(iigs, g0, g1);
    if (ix1 < ix0 || iy1 < iy0) {
        if (!ladd) gf_set(iigs, 0.0, u, ik, igs);
        return;
    }
    int fmx = opt_fft_size(ix1 - ix0 + 1), fmy = opt_fft_size(iy1 - iy0 + 1);
    int NX = 2 * fmx, NY = 2 * fmy;
    if (c.fft_mx != fmx || c.fft_my != fmy) { c.invalidate_fft(); c.fft_mx = fmx; c.fft_my = fmy; }
    if (!c.fft_ok[ik - 1][jk - 1]) {
        std::vector<cplx> cs((size_t)NX * NY, cplx(0, 0));
        int ly = std::min(fmy, my), lx = std::min(fmx, mx);
        for (int iy = -ly; iy <= ly - 1; iy++)
            for (int ix = -lx; ix <= lx - 1; ix++)
                cs[(size_t)(ix + fmx) + (size_t)(iy + fmy) * NX] = c.at(ix, iy, ik, jk);
        fft2d(cs, NX, NY, false);
        c.fft_cf[ik - 1][jk - 1] = std::move(cs);
        c.fft_ok[ik - 1][jk - 1] = true;
    }
    const double *pv = p.col(jk);
    const std::vector<cplx> &cf = c.fft_cf[ik - 1][jk - 1];
#ifdef ORC_FAST_FFT
    // baseline build: the same product by real-input transforms
    std::vector<double> pr((size_t)NX * NY, 0.0), ur((size_t)NX * NY);
    for (int iy = iy0; iy <= iy1; iy++)
        for (int ix = ix0; ix <= ix1; ix++)
            pr[(size_t)(ix - ix0) + (size_t)(iy - iy0) * NX] = pv[(ix - 1) + (iy - 1) * mx];
    real_conv2d(pr.data(), cf.data(), NX, NY, ur.data());
    auto result = [&](size_t q) { return ur[q]; };
#else
    std::vector<cplx> ps((size_t)NX * NY, cplx(0, 0));
    for (int iy = iy0; iy <= iy1; iy++)
        for (int ix = ix0; ix <= ix1; ix++)
            ps[(size_t)(ix - ix0) + (size_t)(iy - iy0) * NX] = pv[(ix - 1) + (iy - 1) * mx];
    fft2d(ps, NX, NY, false);
    for (size_t k = 0; k < ps.size(); k++) ps[k] *= cf[k];
    fft2d(ps, NX, NY, true);
    auto result = [&](size_t q) { return ps[q].real(); };
#endif
    const double scale = 1.0 / (4.0 * fmx * fmy);
    double *uv = u.col(ik);
    for (int iy = iy0; iy <= iy1; iy++)
        for (int ix = ix0; ix <= ix1; ix++) {
            int ii = (ix - 1) + (iy - 1) * mx;
            if (igs.el[ii] >= g0 && igs.el[ii] <= g1) {
                double val = result((size_t)(fmx + ix - ix0) + (size_t)(fmy + iy - iy0) * NX) * scale;
                uv[ii] = ladd ? uv[ii] + val : val;
            }
        }
}

// gf3_VecAijPj, m_aijpj.f90:258-451 (FFT branch, with the M=4 layer term; B=1 is not restated)
inline void vecaijpj(const Eldiv &igs, int iigs, GF3 &u, int ikarg, const GF3 &p, const Eldiv &pe,
                     int jkarg, Inflcf &c, int mx, int my) {
    int ik0, ik1, jk0, jk1;
    ikrange(ikarg, ik0, ik1);
    if (jkarg == -3) { jk0 = 1; jk1 = 3; }
    else if (jkarg == -2) { jk0 = 1; jk1 = 2; }
    else if (jkarg >= 1 && jkarg <= 3) { jk0 = jk1 = jkarg; }
    else { jk0 = 1; jk1 = 0; }
    for (int ik = ik0; ik <= ik1; ik++) {
        bool ladd = false;
        for (int jk = jk0; jk <= jk1; jk++) {
            if (!c.nt_cpl && (ik * jk == 3 || ik * jk == 6)) {
                if (!ladd) gf_set(iigs, 0.0, u, ik, igs);
            } else {
                fft_vecaijpj(igs, ladd, iigs, u, ik, p, pe, jk, c, mx, my);
                ladd = true;
            }
        }
    }
    gf_scal(iigs, c.ga_inv, u, ikarg, igs);
    if (c.use_3bl) {                              // m_aijpj.f90:409-421
        int g0, g1;
        igsrange(iigs, g0, g1);
        for (int ik = ik0; ik <= std::min(ik1, (int)ikY); ik++) {
            if (!(jkarg == ik || jkarg <= ikTANG)) continue;
            double *uv = u.col(ik);
            const double *pv = p.col(ik);
            for (int ii = 0; ii < (int)igs.el.size(); ii++)
                if (igs.el[ii] >= g0 && igs.el[ii] <= g1) uv[ii] += c.flx_3bl * pv[ii];
        }
    }
}

// fft_makePrec, m_aijpj.f90:457-708: m = ga^2 * IFFT(1 ./ FFT(c)) on the cf window
inline void fft_makeprec(int ik, Inflcf &c, int jk, Inflcf &m) {
    m.nt_cpl = c.nt_cpl;
    int fmx = c.cf_mx, fmy = c.cf_my;
    int NX = 2 * fmx, NY = 2 * fmy;
    if (c.fft_mx != fmx || c.fft_my != fmy) { c.invalidate_fft(); c.fft_mx = fmx; c.fft_my = fmy; }
    if (!c.fft_ok[ik - 1][jk - 1]) {
        std::vector<cplx> cs((size_t)NX * NY, cplx(0, 0));
        for (int iy = -fmy; iy <= fmy - 1; iy++)
            for (int ix = -fmx; ix <= fmx - 1; ix++)
                cs[(size_t)(ix + fmx) + (size_t)(iy + fmy) * NX] = c.at(ix, iy, ik, jk);
        fft2d(cs, NX, NY, false);
        c.fft_cf[ik - 1][jk - 1] = std::move(cs);
        c.fft_ok[ik - 1][jk - 1] = true;
    }
    const std::vector<cplx> &cf = c.fft_cf[ik - 1][jk - 1];
    std::vector<cplx> mf(cf.size());
    for (size_t k = 0; k < cf.size(); k++) mf[k] = 1.0 / cf[k];
    fft2d(mf, NX, NY, true);
    const double scale = 1.0 / (4.0 * fmx * fmy);
    for (int iy = -fmy; iy <= fmy - 1; iy++)
        for (int ix = -fmx; ix <= fmx - 1; ix++)
            m.at(ix, iy, ik, jk) = c.ga * c.ga * mf[(size_t)(ix + fmx) + (size_t)(iy + fmy) * NX].real() * scale;
    m.invalidate_fft();
}

} // namespace orc
