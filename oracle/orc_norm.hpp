// CPU ORACLE -- test infrastructure only (see contact_oracle.h).
//
// Normal problem: snorm (m_snorm.f90:31-378) around normcg (m_solvpn.f90:24-461).
#pragma once
#include "orc_conv.hpp"

namespace orc {

struct NormCtx {
    int mx, my, npot;
    double dxdy;
    int ic_norm;           // N digit
    double fntrue;
};

// normcg, m_solvpn.f90:24-461.  Returns itcg; err out.  Sets 'abort' when the reference
// would stop the program (divergence past maxcg, m_solvpn.f90:423-429).
inline int normcg(const NormCtx &cx, bool use_fftprec, int maxcg, double eps, Inflcf &cs, Inflcf &ms,
                  const GF3 &hstot, double &pen, Eldiv &igs, GF3 &ps, double &err, bool &abort,
                  bool is_sens = false) {
    const int mx = cx.mx, my = cx.my, npot = cx.npot;
    const double dxdy = cx.dxdy, fntrue = cx.fntrue;
    abort = false;
    // is_sens: the stopping tolerance is relative to the change from the initial estimate
    // (m_solvpn.f90:92-97, 281-290)
    GF3 ps0, tmp1;
    if (is_sens) { ps0 = ps; tmp1.init(npot); }
    int numinn = (npot <= 150) ? 3 : (npot <= 400) ? 2 : 1;
    GF3 rhs, res, r_prv, dd, z, v, q;
    for (GF3 *g : {&rhs, &res, &r_prv, &dd, &z, &v, &q}) g->init(npot);
    if (cx.ic_norm == 1) pen = 0.0;
    gf_set(AllElm, pen, rhs, ikZ, igs);
    gf_axpy(AllElm, -1.0, hstot, rhs, ikZ, igs);
    double davg = 0.0;
    int ncon = 0;
    for (int i = 0; i < npot; i++) if (igs.el[i] >= Adhes) ncon++;
    int itcg = 0;
    double hsmin, hsmax;
    if (cx.ic_norm == 0) {
        hsmin = gf_min(AllElm, hstot, ikZ, igs) - pen;
        if (hsmin >= 0.0) {
            gf_set(AllElm, 0.0, ps, ikZ, igs);
            for (int i = 0; i < npot; i++) igs.el[i] = Exter;
            err = 0.0;
            return 0;
        }
    } else {
        if (ncon <= 0) {
            hsmin = gf_min(AllElm, hstot, ikZ, igs);
            hsmax = gf_max(AllElm, hstot, ikZ, igs);
            double htrsh = hsmin + 0.1 * std::max(hsmax - hsmin, 1e-10);
            for (int i = 0; i < npot; i++)
                if (hstot.c[2][i] < htrsh) { igs.el[i] = Adhes; ncon++; }
            areas(igs);
        }
        double fk = dxdy * gf_sum(AllElm, ps, ikZ, igs);
        if (std::fabs(fk) < (double)1e-3f * fntrue) {
            double pn = fntrue / (dxdy * (double)(float)ncon);
            gf_set(AllInt, pn, ps, ikZ, igs);
            fk = dxdy * gf_sum(AllElm, ps, ikZ, igs);
        } else {
            gf_scal(AllInt, fntrue / fk, ps, ikZ, igs);
        }
    }
    // res = rhs - A ps
    vecaijpj(igs, AllInt, res, ikZ, ps, igs, ikZ, cs, mx, my);
    gf_scal(AllInt, -1.0, res, ikZ, igs);
    gf_axpy(AllInt, 1.0, rhs, res, ikZ, igs);
    if (cx.ic_norm == 1) gf_proj_avg(AllInt, res, ikZ, igs);
    double rz1 = 0, rz2 = 0.0, rms_upd1 = 0, alpha = 0;
    int itchg = 0, itinn = 0;
    double rms_xk = 1.0, rms_upd = 2.0 * eps * rms_xk;
    bool lchanged = false;
    while ((lchanged || rms_upd > eps * rms_xk) && itcg < maxcg) {
        itcg++; itinn++;
        if (use_fftprec) vecaijpj(igs, AllInt, z, ikZ, res, igs, ikZ, ms, mx, my);
        else gf_copy(AllElm, res, z, ikZ, igs);
        if (cx.ic_norm == 1) gf_proj_avg(AllInt, z, ikZ, igs);
        rz1 = rz2;
        rz2 = gf_dot(AllInt, z, res, ikZ, igs);
        if (itcg <= 1 || rz1 < tiny_) {
            gf_copy(AllInt, z, v, ikZ, igs);
        } else {
            double rrprv = gf_dot(AllInt, z, r_prv, ikZ, igs);
            double beta = std::max(0.0, (rz2 - rrprv) / std::max(tiny_, rz1));
            gf_scal(AllInt, beta, v, ikZ, igs);
            gf_axpy(AllInt, 1.0, z, v, ikZ, igs);
        }
        if (cx.ic_norm == 1) gf_proj_avg(AllInt, v, ikZ, igs);
        vecaijpj(igs, AllInt, q, ikZ, v, igs, ikZ, cs, mx, my);
        if (cx.ic_norm == 1) gf_proj_avg(AllInt, q, ikZ, igs);
        double rv = gf_dot(AllInt, res, v, ikZ, igs);
        double vav = gf_dot(AllInt, q, v, ikZ, igs);
        if (std::fabs(vav) > 1e-32 && ncon == 1) alpha = rv / vav;
        else alpha = rv / std::max(tiny_, vav);
        gf_axpy(AllInt, alpha, v, ps, ikZ, igs);
        rms_upd = std::fabs(alpha) * gf_rms(AllInt, v, ikZ, igs);
        if (itcg == 1) rms_upd1 = rms_upd;
        if (itcg <= 3 || itcg % 10 == 0) {
            if (!is_sens) {
                rms_xk = gf_rms(AllInt, ps, ikZ, igs);
            } else {
                gf_copy(AllElm, ps, tmp1, ikZ, igs);
                gf_axpy(AllElm, -1.0, ps0, tmp1, ikZ, igs);
                rms_xk = gf_rms(AllInt, tmp1, ikZ, igs);
            }
        }
        gf_copy(AllElm, res, r_prv, ikZ, igs);
        if (itinn < numinn && rms_upd >= eps * rms_xk) {
            gf_axpy(AllInt, -alpha, q, res, ikZ, igs);
        } else {
            bool lchg_negpn = false;
            for (int i = 0; i < npot; i++)
                if (igs.el[i] >= Adhes && ps.c[2][i] < 0.0) {
                    igs.el[i] = Exter; ncon--; ps.c[2][i] = 0.0; lchg_negpn = true;
                }
            if (ncon <= 0) {
                hsmin = gf_min(AllElm, hstot, ikZ, igs);
                for (int i = 0; i < npot; i++)
                    if (hstot.c[2][i] <= hsmin + 1e-5) {
                        igs.el[i] = Adhes; ncon++; ps.c[2][i] = 0.0; lchg_negpn = true;
                    }
            }
            if (cx.ic_norm == 1 && lchg_negpn) {
                double fk = dxdy * gf_sum(AllElm, ps, ikZ, igs);
                if (std::fabs(fk) < (double)1e-3f * fntrue) {
                    gf_set(AllInt, 1.0, ps, ikZ, igs);
                    fk = gf_sum(AllElm, ps, ikZ, igs);
                }
                gf_scal(AllInt, fntrue / fk, ps, ikZ, igs);
            }
            if (lchg_negpn) areas(igs);
            vecaijpj(igs, AllElm, dd, ikZ, ps, igs, ikZ, cs, mx, my);
            gf_axpy(AllElm, -1.0, rhs, dd, ikZ, igs);
            if (cx.ic_norm == 1) {
                davg = gf_sum(AllInt, dd, ikZ, igs) / (double)(float)ncon;
                gf_proj_avg(AllInt, dd, ikZ, igs);
            }
            gf_set(AllElm, 0.0, res, ikZ, igs);
            gf_axpy(AllInt, -1.0, dd, res, ikZ, igs);
            bool lchg_intpen = false;
            for (int i = 0; i < npot; i++)
                if (igs.el[i] == Exter && dd.c[2][i] - davg < 0.0) {
                    igs.el[i] = Adhes; ncon++; res.c[2][i] = -(dd.c[2][i] - davg); lchg_intpen = true;
                }
            for (int i = 0; i < npot; i++) if (igs.el[i] == Exter) v.c[2][i] = 0.0;
            if (lchg_intpen) areas(igs);
            itinn = 0;
            lchanged = lchg_intpen || lchg_negpn;
            if (lchanged) itchg++;
        }
    }
    if (cx.ic_norm == 1) pen = davg;
    double conv = 1.0;
    if (rms_upd * rms_upd1 > 0.0 && itcg > 1) conv = std::exp(std::log(rms_upd / rms_upd1) / (itcg - 1));
    if (rms_upd > rms_xk && conv > 1.0 && itcg >= maxcg) abort = true;
    err = rms_upd;
    return itcg;
}

// sens_norm, m_solvpn.f90:531-650: d Fn / d pen from one NormCG solve with the approach
// perturbed by 0.67 % of the largest normal displacement, started from the solution.
// Returns false when that solve diverges (the reference stops there).
inline bool sens_norm(const NormCtx &cx, int mxsens, double epsens, Inflcf &cs, Inflcf &ms,
                      const GF3 &hstot, double pen, double fntrue, const Eldiv &igs, const GF3 &ps,
                      const GF3 &unn, double &sens_fn_pen) {
    NormCtx loc = cx;
    loc.ic_norm = 0;
    double pentru = gf_max(AllInt, unn, ikZ, igs);
    double dpen = 0.0067 * pentru;
    double penloc = pen + dpen;
    Eldiv igsloc = igs;
    GF3 psloc; psloc.init(cx.npot);
    gf_copy(AllElm, ps, psloc, ikZ, igsloc);
    double err; bool abort;
    normcg(loc, true, mxsens, epsens, cs, ms, hstot, penloc, igsloc, psloc, err, abort, true);
    if (abort) return false;
    double fnloc = cx.dxdy * gf_sum(AllElm, psloc, ikZ, igsloc);
    sens_fn_pen = (fnloc - fntrue) / dpen;
    return true;
}

// snorm, m_snorm.f90:31-378.  Returns itnorm (-1: maxin reached, -2: normcg divergence).
// sens >= 2 adds d Fn / d pen (m_snorm.f90:357-368) into sens_fn_pen, else sets it to zero.
inline int snorm(const NormCtx &cx, int maxgs, int maxin, double eps, Inflcf &cs, Inflcf &ms,
                 const GF3 &hs, double &pen, Eldiv &igs1, GF3 &ps1, int &itcg_out,
                 int sens = 1, int mxsens = 30, double epsens = 1e-4, double *sens_fn_pen = nullptr) {
    const int mx = cx.mx, my = cx.my, npot = cx.npot;
    areas(igs1);
    bool use_vecfft = (npot >= 700);
    bool use_fftprec = true;
    if (use_fftprec) fft_makeprec(3, cs, 3, ms);
    GF3 htang, hstot, tmp, unn;
    for (GF3 *g : {&htang, &hstot, &tmp, &unn}) g->init(npot);
    gf_copy(AllElm, hs, hstot, ikZ, igs1);
    if (cs.nt_cpl) {
        vecaijpj(igs1, AllElm, htang, ikZ, ps1, igs1, ikTANG, cs, mx, my);
        gf_axpy(AllElm, 1.0, htang, hstot, ikZ, igs1);
    }
    int itnorm = 0, itcg = 0;
    bool zready;
    int ncon = 0;
    do {
        itnorm++;
        zready = true;
        ncon = 0;
        for (int i = 0; i < npot; i++) {
            if (igs1.el[i] >= Adhes) ncon++; else ps1.c[2][i] = 0.0;
        }
        areas(igs1);
        double errpn; bool abort;
        int it = normcg(cx, use_fftprec, maxgs, eps, cs, ms, hstot, pen, igs1, ps1, errpn, abort);
        if (abort) { itcg_out = itcg + it; return -2; }
        itcg += it;
        ncon = 0;
        for (int i = 0; i < npot; i++) if (igs1.el[i] >= Adhes) ncon++;
        int newext = 0;
        for (int i = 0; i < npot; i++)
            if (igs1.el[i] >= Adhes && ps1.c[2][i] < -errpn) { igs1.el[i] = Exter; newext++; ps1.c[2][i] = 0.0; }
        ncon -= newext;
        if (newext > 0) zready = false;
        if (zready) {
            areas(igs1);
            if (use_vecfft) vecaijpj(igs1, AllElm, unn, ikZ, ps1, igs1, ikZ, cs, mx, my);
            int ix = std::max(1, mx / 2), iy = std::max(1, my / 2);
            int ii = (ix - 1) + (iy - 1) * mx;
            gf_set(AllElm, 1.0, tmp, ikZ, igs1);
            double tol = std::fabs(errpn * aijpj(ii, ikZ, tmp, igs1, ikZ, cs, mx, my));
            int newcon = 0;
            for (int i = 0; i < npot; i++) {
                if (igs1.el[i] == Exter && hstot.c[2][i] - pen < 0.0) {
                    double dd;
                    if (use_vecfft) dd = hstot.c[2][i] - pen + unn.c[2][i];
                    else dd = hstot.c[2][i] - pen + aijpj(i, ikZ, ps1, igs1, ikZ, cs, mx, my);
                    if (dd < -tol) { igs1.el[i] = Adhes; newcon++; }
                }
            }
            ncon += newcon;
            if (newcon != 0) zready = false;
        }
        if (it >= maxgs) zready = false;
    } while (!zready && itnorm < maxin);
    if (!zready) itnorm = -1;
    for (int i = 0; i < npot; i++)
        if (ps1.c[2][i] < 0.0 && igs1.el[i] >= Adhes) { ps1.c[2][i] = 0.0; igs1.el[i] = Exter; }
    areas(igs1);
    itcg_out = itcg;
    if (sens_fn_pen) {
        if (sens >= 2) {
            double fntrue = cx.fntrue;
            if (cx.ic_norm == 0) fntrue = cx.dxdy * gf_sum(AllElm, ps1, ikZ, igs1);
            if (!use_vecfft) vecaijpj(igs1, AllElm, unn, ikZ, ps1, igs1, ikZ, cs, mx, my);
            if (!sens_norm(cx, mxsens, epsens, cs, ms, hstot, pen, fntrue, igs1, ps1, unn, *sens_fn_pen))
                return -2;
        } else {
            *sens_fn_pen = 0.0;
        }
    }
    return itnorm;
}

} // namespace orc
