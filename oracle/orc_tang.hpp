// CPU ORACLE -- test infrastructure only (see contact_oracle.h).
//
// Tangential problem: stang (m_stang.f90:28-746), stang_rhs (:749-951), leading edge
// sxbnd and subnd (m_leadedge.f90:92-394), the solvers SteadyGS (m_solvpt.f90:2825-3254),
// ConvexGS (m_solvpt.f90:2446-2821), GDsteady (gdsteady.f90:9-1462) and TangCG
// (m_solvpt.f90:1841-2442).
#pragma once
#include "orc_conv.hpp"
#include "orc_elm.hpp"

namespace orc {

struct TangCtx {
    int mx, my, npot;
    double dx, dy, dxdy;
    int tang;                 // T digit
    double chi, dq;
    int gausei_eff;           // effective G digit
    int maxgs, maxin;
    double eps;
    double omegah, omegas;
    int gd_meth, kdown, kdowfb;
    double fdecay, betath, d_ifc, d_lin, d_cns, d_slp, pow_s;
};

// Leading edge of the contact area (t_leadedge, m_leadedge.f90:20-70): per row iy the
// positions jbnd[iy-1] .. jbnd[iy]-1 (1-based), their last interior column ixbnd, their
// relative offset facdx to the edge and the rolling direction ixinc
struct Ledg {
    std::vector<int> jbnd, ixbnd;
    std::vector<double> facdx;
    int ixinc = 1;
};

// sxbnd, m_leadedge.f90:92-332: facdt per element, leading edge index map ii2j (0 = none)
inline void sxbnd(const TangCtx &cx, int solver_eff, const Eldiv &igs, const Grid &g,
                  std::vector<double> &facdt, std::vector<int> &ii2j, Ledg *ledg = nullptr) {
    const int mx = cx.mx, my = cx.my;
    bool is_roll = cx.tang == 2 || cx.tang == 3;
    int ixsta, ixinc, ixend;
    if (is_roll && std::fabs(cx.chi - pi) < 0.01) { ixsta = mx; ixinc = -1; ixend = 1; }
    else { ixsta = 1; ixinc = 1; ixend = mx; }
    std::vector<int> jbnd(my + 1), ixbnd;
    jbnd[0] = 1;
    for (int iy = 1; iy <= my; iy++) {
        int npos = 0;
        for (int ix = ixsta; ix != ixend; ix += ixinc) {
            int ii = (ix - 1) + (iy - 1) * mx;
            if (igs.el[ii] >= Adhes && igs.el[ii + ixinc] <= Exter) npos++;
        }
        if (igs.el[(ixend - 1) + (iy - 1) * mx] >= Adhes) npos++;
        jbnd[iy] = jbnd[iy - 1] + npos;
    }
    int npos = jbnd[my];
    ixbnd.assign(npos + 1, 0);
    for (int iy = 1; iy <= my; iy++) {
        if (jbnd[iy] - jbnd[iy - 1] > 0) {
            int j = jbnd[iy - 1];
            for (int ix = ixsta; ix != ixend; ix += ixinc) {
                int ii = (ix - 1) + (iy - 1) * mx;
                if (igs.el[ii] >= Adhes && igs.el[ii + ixinc] <= Exter) ixbnd[j++] = ix;
            }
            if (igs.el[(ixend - 1) + (iy - 1) * mx] >= Adhes) ixbnd[j++] = ixend;
        }
    }
    bool use_ledg = (solver_eff != isolv_stdygs);
    double fxdfac = use_ledg ? 1.0 : 2.0;
    std::vector<double> xbnd(npos + 1, 0.0);
    for (int iy = 1; iy <= my; iy++)
        for (int j = jbnd[iy - 1]; j <= jbnd[iy] - 1; j++) {
            int ii = (ixbnd[j] - 1) + (iy - 1) * mx;
            xbnd[j] = g.x[ii] + ixinc * fxdfac * g.dx;
        }
    facdt.assign(cx.npot, 0.0);
    ii2j.assign(cx.npot, 0);
    for (int iy = 1; iy <= my; iy++) {
        int j = jbnd[iy - 1];
        for (int ix = ixsta; ; ix += ixinc) {
            while (j < jbnd[iy] && ((ixinc > 0 && ix > ixbnd[j]) || (ixinc < 0 && ix < ixbnd[j]))) j++;
            int ii = (ix - 1) + (iy - 1) * mx;
            if (!is_roll) { ii2j[ii] = 0; facdt[ii] = 1.0; }
            else if (igs.el[ii] <= Exter) { ii2j[ii] = 0; facdt[ii] = 0.0; }
            else if ((ixinc > 0 && ix + 2 > mx) || (ixinc < 0 && ix - 2 <= 0)) { ii2j[ii] = 0; facdt[ii] = 1.0; }
            else {
                facdt[ii] = std::min(1.0, ixinc * (xbnd[j] - g.x[ii]) / cx.dq);
                ii2j[ii] = (facdt[ii] < 0.9999) ? j : 0;
            }
            if (ix == ixend) break;
        }
    }
    if (ledg) {
        ledg->jbnd = jbnd;
        ledg->ixbnd = ixbnd;
        ledg->facdx.assign(npos + 1, fxdfac);
        ledg->ixinc = ixinc;
    }
}

// subnd, m_leadedge.f90:336-394: the tangential displacement difference at each leading edge
// position, interpolated between its last interior element and the next one; zero where the
// edge is within two elements of the grid's end
inline void subnd(const TangCtx &cx, const Ledg &L, const GF3 &p, const Eldiv &pe, const Inflcf &c,
                  std::vector<double> &ubnd) {
    const int mx = cx.mx, my = cx.my, ixinc = L.ixinc;
    const int npos = L.jbnd[my];
    ubnd.assign((size_t)2 * (npos + 1), 0.0);
    for (int iy = 1; iy <= my; iy++)
        for (int j = L.jbnd[iy - 1]; j <= L.jbnd[iy] - 1; j++) {
            const int ix0 = L.ixbnd[j];
            if ((ixinc > 0 && ix0 + 2 > mx) || (ixinc < 0 && ix0 - 2 <= 0)) continue;
            const int ii = (ix0 - 1) + (iy - 1) * mx;
            for (int ik = 1; ik <= 2; ik++) {
                const double u0 = aijpj(ii, ik, p, pe, -3, c, mx, my);
                const double u1 = aijpj(ii + ixinc, ik, p, pe, -3, c, mx, my);
                ubnd[(size_t)2 * j + ik - 1] = (1.0 - L.facdx[j]) * u0 + L.facdx[j] * u1;
            }
        }
}

// ------------------------------------------------------------------------------------------
// SteadyGS, m_solvpt.f90:2825-3254 (no plasticity: taucs never limits the bound)
// ------------------------------------------------------------------------------------------
inline int stdygs(const TangCtx &cx, const GF3 &ws, Inflcf &cs, Eldiv &igs, const std::vector<double> &mus,
                  GF3 &ps, GF3 &ss, double eps, int maxgs, double omegah, double omegas,
                  int &info, double &err, bool &bad, bool is_sens = false) {
    const int mx = cx.mx, my = cx.my, npot = cx.npot;
    bad = false;
    const double flx = cs.use_3bl ? cs.flx_3bl : 0.0;     // m_solvpt.f90:2922-2929
    int ixsta, ixinc, ixend;
    // is_sens: the stopping tolerance is relative to the change from the initial estimate
    // (m_solvpt.f90:2893-2899, 3138-3145)
    GF3 ps0, tmp;
    if (is_sens) { ps0 = ps; tmp.init(npot); }
    if (std::fabs(cx.chi) < 0.01) { ixsta = 1; ixinc = 1; ixend = mx; }
    else if (std::fabs(cx.chi - pi) < 0.01) { ixsta = mx; ixinc = -1; ixend = 1; }
    else { bad = true; return 0; }
    GF3 dp; dp.init(npot);
    for (int iy = 1; iy <= my; iy++)
        for (int ix = 1; ix <= mx; ix++) {
            int ii = (ix - 1) + (iy - 1) * mx;
            if (ix != ixend) {
                dp.vx(ii) = ps.c[0][ii] - ps.c[0][ii + ixinc];
                dp.vy(ii) = ps.c[1][ii] - ps.c[1][ii + ixinc];
            } else {
                dp.vx(ii) = ps.c[0][ii]; dp.vy(ii) = ps.c[1][ii];
            }
        }
    int nadh, nslip, nplst, nexter;
    eldiv_count(igs, nadh, nslip, nplst, nexter);
    int k = nadh + nslip + nplst;
    double facnel = std::sqrt((double)(float)npot / (double)(float)(nadh + nslip + nplst));
    int itgs = 0;
    double dif = 2.0, difid = 1.0, dif1 = 0.0;
    while (dif >= difid && itgs < maxgs) {
        itgs++;
        dif = 0.0;
        for (int iy = 1; iy <= my; iy++) {
            int ix = ixsta - ixinc;
            while (ix != ixend) {
                ix += ixinc;
                int ii = (ix - 1) + (iy - 1) * mx;
                if (igs.el[ii] < Adhes) continue;
                int jx = ix - ixinc;
                int jj = (jx - 1) + (iy - 1) * mx;
                while (igs.el[jj] == Adhes && jx != ixsta) { jx -= ixinc; jj = (jx - 1) + (iy - 1) * mx; }
                double coef[2][2];
                coef[0][0] = cs.ga_inv * (cs.at(0, 0, 1, 1) - cs.at(jx - ix, 0, 1, 1)) + flx;
                coef[0][1] = cs.ga_inv * (cs.at(0, 0, 1, 2) - cs.at(jx - ix, 0, 1, 2));
                coef[1][0] = cs.ga_inv * (cs.at(0, 0, 2, 1) - cs.at(jx - ix, 0, 2, 1));
                coef[1][1] = cs.ga_inv * (cs.at(0, 0, 2, 2) - cs.at(jx - ix, 0, 2, 2)) + flx;
                double s[2];
                s[0] = ws.c[0][ii] + aijpj(ii, ikX, dp, igs, ikTANG, cs, mx, my);
                s[1] = ws.c[1][ii] + aijpj(ii, ikY, dp, igs, ikTANG, cs, mx, my);
                double pr[3] = {ps.c[0][ii], ps.c[1][ii], ps.c[2][ii]};
                double taucs = 0.0, dupl[2];
                int el = igs.el[ii];
                plstrc(el, coef, eps, omegah, omegas, pr, mus[ii], false, 0.0, 0.0, 0.0, taucs, s, dupl);
                igs.el[ii] = el;
                dif += (pr[0] - ps.c[0][ii]) * (pr[0] - ps.c[0][ii]) + (pr[1] - ps.c[1][ii]) * (pr[1] - ps.c[1][ii]);
                dp.vx(ii) = dp.vx(ii) + pr[0] - ps.c[0][ii];
                dp.vy(ii) = dp.vy(ii) + pr[1] - ps.c[1][ii];
                ps.c[0][ii] = pr[0]; ps.c[1][ii] = pr[1];
                ss.c[0][ii] = s[0]; ss.c[1][ii] = s[1];
                // propagate the change of dp(ii) towards the trailing edge
                for (int kx = ix - ixinc; ; kx -= ixinc) {
                    if ((ixinc > 0 && kx < ixsta) || (ixinc < 0 && kx > ixsta)) break;
                    int kk = (kx - 1) + (iy - 1) * mx;
                    int kn = kk + ixinc;
                    if (igs.el[kk] == Adhes) {
                        ps.c[0][kk] = ps.c[0][kn] + dp.vx(kk);
                        ps.c[1][kk] = ps.c[1][kn] + dp.vy(kk);
                        double ptabs = std::sqrt(ps.c[0][kk] * ps.c[0][kk] + ps.c[1][kk] * ps.c[1][kk]);
                        double ptbnd = mus[kk] * ps.c[2][kk];
                        if (ptabs > ptbnd) {
                            ps.c[0][kk] = ps.c[0][kk] * ptbnd / ptabs;
                            ps.c[1][kk] = ps.c[1][kk] * ptbnd / ptabs;
                            dp.vx(kk) = ps.c[0][kk] - ps.c[0][kn];
                            dp.vy(kk) = ps.c[1][kk] - ps.c[1][kn];
                        }
                    } else if (igs.el[kk] == Slip || igs.el[kk] == Plast) {
                        dp.vx(kk) = ps.c[0][kk] - ps.c[0][kn];
                        dp.vy(kk) = ps.c[1][kk] - ps.c[1][kn];
                    } else if (igs.el[kk] <= Exter && igs.el[kn] >= Adhes) {
                        dp.vx(kk) = -ps.c[0][kn];
                        dp.vy(kk) = -ps.c[1][kn];
                    }
                }
            }
        }
        dif = std::sqrt(dif / (2.0 * k));
        if (!is_sens) {
            difid = eps * std::max(1e-6, facnel * gf_rms(AllElm, ps, ikTANG, igs));
        } else {
            gf_copy(AllElm, ps, tmp, ikTANG, igs);
            gf_axpy(AllElm, -1.0, ps0, tmp, ikTANG, igs);
            difid = eps * std::max(1e-6, facnel * gf_rms(AllElm, tmp, ikTANG, igs));
        }
        if (itgs == 1) dif1 = dif;
    }
    double conv = 1.0;
    if (dif * dif1 != 0.0 && itgs > 1) conv = std::exp(std::log(dif / dif1) / (itgs - 1));
    err = dif;
    info = 0;
    if (itgs >= maxgs) info = 1;
    if (itgs >= maxgs && conv > 0.997) info = 2;
    if (itgs >= maxgs && conv > 1.0) info = 3;
    return itgs;
}

// ------------------------------------------------------------------------------------------
// ConvexGS, m_solvpt.f90:2446-2821 (elastic, no third-body layer): block Gauss-Seidel over the
// contact elements in the order of iel (reversed for chi = pi) with the element solver plstrc.
// Shifts per element from the current tractions: cs for shifts and transient rolling (T=1, 2);
// for steady rolling (T=3) csv = cs - cv (the displacement difference of one rolling step), or
// near the leading edge cs minus the edge estimate ubnd (subnd, refreshed every sweep).
// ------------------------------------------------------------------------------------------
inline int cnvxgs(const TangCtx &cx, const GF3 &ws, Inflcf &cs, const Inflcf *csv, const Ledg &L,
                  const std::vector<int> &ii2j, const std::vector<int> &iel, Eldiv &igs,
                  const std::vector<double> &mus, GF3 &ps, GF3 &ss, double eps, int maxgs, double omegah,
                  double omegas, int &info, double &err, bool is_sens = false) {
    const int mx = cx.mx, my = cx.my, npot = cx.npot, k = (int)iel.size();
    const bool is_ssrol = cx.tang == 3;
    if (k == 0) { info = 0; err = 0.0; return 0; }
    GF3 ps0, tmp;
    if (is_sens) { ps0 = ps; tmp.init(npot); }
    int ista, iinc, iend;
    if (std::fabs(cx.chi - pi) < 0.01) { ista = k - 1; iinc = -1; iend = 0; }
    else { ista = 0; iinc = 1; iend = k - 1; }
    double coefs[2][2], coefsv[2][2];
    const double flx = cs.use_3bl ? cs.flx_3bl : 0.0;     // m_solvpt.f90:2523-2552
    coefs[0][0] = cs.ga_inv * cs.at(0, 0, 1, 1) + flx; coefs[0][1] = cs.ga_inv * cs.at(0, 0, 1, 2);
    coefs[1][0] = cs.ga_inv * cs.at(0, 0, 2, 1); coefs[1][1] = cs.ga_inv * cs.at(0, 0, 2, 2) + flx;
    const Inflcf &cv = csv ? *csv : cs;
    coefsv[0][0] = cv.ga_inv * cv.at(0, 0, 1, 1) + flx; coefsv[0][1] = cv.ga_inv * cv.at(0, 0, 1, 2);
    coefsv[1][0] = cv.ga_inv * cv.at(0, 0, 2, 1); coefsv[1][1] = cv.ga_inv * cv.at(0, 0, 2, 2) + flx;
    int nadh, nslip, nplst, nexter;
    eldiv_count(igs, nadh, nslip, nplst, nexter);
    const double facnel = std::sqrt((double)(float)npot / (double)(float)(nadh + nslip + nplst));
    int itgs = 0;
    double dif = 2.0, difid = 1.0, dif1 = 0.0;
    std::vector<double> ubnd;
    while (dif >= difid && itgs < maxgs) {
        itgs++;
        dif = 0.0;
        if (is_ssrol) subnd(cx, L, ps, igs, cs, ubnd);
        for (int i = ista; ; i += iinc) {
            const int ii = iel[i];
            if (itgs <= 1000 || itgs % 2 == 0 || igs.el[ii] == Adhes) {
                double pr[3] = {ps.c[0][ii], ps.c[1][ii], ps.c[2][ii]};
                double dupl[2] = {0.0, 0.0}, taucs = 0.0;
                const bool zledge = is_ssrol && ii2j[ii] > 0;
                double s[2];
                if (!is_ssrol) {
                    s[0] = ws.c[0][ii] + aijpj(ii, ikX, ps, igs, ikTANG, cs, mx, my);
                    s[1] = ws.c[1][ii] + aijpj(ii, ikY, ps, igs, ikTANG, cs, mx, my);
                } else if (!zledge) {
                    s[0] = ws.c[0][ii] + aijpj(ii, ikX, ps, igs, ikTANG, cv, mx, my);
                    s[1] = ws.c[1][ii] + aijpj(ii, ikY, ps, igs, ikTANG, cv, mx, my);
                } else {
                    const int j = ii2j[ii];
                    s[0] = ws.c[0][ii] + aijpj(ii, ikX, ps, igs, ikTANG, cs, mx, my) - ubnd[(size_t)2 * j];
                    s[1] = ws.c[1][ii] + aijpj(ii, ikY, ps, igs, ikTANG, cs, mx, my) - ubnd[(size_t)2 * j + 1];
                }
                int el = igs.el[ii];
                plstrc(el, (!is_ssrol || zledge) ? coefs : coefsv, eps, omegah, omegas, pr, mus[ii], false, 0.0, 0.0,
                       0.0, taucs, s, dupl);
                igs.el[ii] = el;
                dif += (ps.c[0][ii] - pr[0]) * (ps.c[0][ii] - pr[0]) + (ps.c[1][ii] - pr[1]) * (ps.c[1][ii] - pr[1]);
                ps.c[0][ii] = pr[0]; ps.c[1][ii] = pr[1];
                ss.c[0][ii] = s[0]; ss.c[1][ii] = s[1];
            }
            if (i == iend) break;
        }
        dif = std::sqrt(dif / (2.0 * k));
        if (!is_sens) {
            difid = eps * std::max(1e-6, facnel * gf_rms(AllElm, ps, ikTANG, igs));
        } else {
            gf_copy(AllElm, ps, tmp, ikTANG, igs);
            gf_axpy(AllElm, -1.0, ps0, tmp, ikTANG, igs);
            difid = eps * std::max(1e-6, facnel * gf_rms(AllElm, tmp, ikTANG, igs));
        }
        if (itgs == 1) dif1 = dif;
    }
    double conv = 1.0;
    if (dif * dif1 != 0.0 && itgs > 1) conv = std::exp(std::log(dif / dif1) / (itgs - 1));
    err = dif;
    info = 0;
    if (itgs >= maxgs) info = 1;
    if (itgs >= maxgs && conv > 0.997) info = 2;
    if (itgs >= maxgs && conv > 1.0) info = 3;
    return itgs;
}

// ------------------------------------------------------------------------------------------
// GDsteady, gdsteady.f90
// ------------------------------------------------------------------------------------------
inline void compute_dp(const GF3 &ps, GF3 &dp, int mx, int my) {   // gdsteady.f90:610-635
    for (int iy = 1; iy <= my; iy++) {
        int ii = (mx - 1) + (iy - 1) * mx;
        dp.c[0][ii] = ps.c[0][ii]; dp.c[1][ii] = ps.c[1][ii];
        for (int ix = mx - 1; ix >= 1; ix--) {
            ii = (ix - 1) + (iy - 1) * mx;
            dp.c[0][ii] = ps.c[0][ii] - ps.c[0][ii + 1];
            dp.c[1][ii] = ps.c[1][ii] - ps.c[1][ii + 1];
        }
    }
}

// apply_trcbnd, gdsteady.f90:807-847
inline void apply_trcbnd(const Eldiv &igs, const std::vector<double> &trcbnd, GF3 &dp, GF3 &ps, int mx, int my) {
    for (int iy = 1; iy <= my; iy++) {
        int ii = (mx - 1) + (iy - 1) * mx;
        ps.c[0][ii] = 0.0; ps.c[1][ii] = 0.0;
        for (int ix = mx - 1; ix >= 1; ix--) {
            ii = (ix - 1) + (iy - 1) * mx;
            if (igs.el[ii] <= Exter) { ps.c[0][ii] = 0.0; ps.c[1][ii] = 0.0; }
            else {
                ps.c[0][ii] = ps.c[0][ii + 1] + dp.c[0][ii];
                ps.c[1][ii] = ps.c[1][ii + 1] + dp.c[1][ii];
                double ptabs = std::sqrt(ps.c[0][ii] * ps.c[0][ii] + ps.c[1][ii] * ps.c[1][ii]);
                if (igs.el[ii] == Slip || ptabs >= trcbnd[ii]) {
                    ps.c[0][ii] = ps.c[0][ii] * trcbnd[ii] / ptabs;
                    ps.c[1][ii] = ps.c[1][ii] * trcbnd[ii] / ptabs;
                }
            }
            dp.c[0][ii] = ps.c[0][ii] - ps.c[0][ii + 1];
            dp.c[1][ii] = ps.c[1][ii] - ps.c[1][ii + 1];
        }
    }
}

inline double fsign(double a, double b) { return b >= 0.0 ? std::fabs(a) : -std::fabs(a); }

// project_searchdir, gdsteady.f90:639-803
inline void project_searchdir(const TangCtx &cx, const Eldiv &igs, const std::vector<double> &trcbnd, int itgd,
                              int &it_fb, double betaj, const GF3 &t, GF3 &dv, GF3 &v, double fac_v) {
    const int mx = cx.mx, my = cx.my;
    int imeth, kdown;
    if (betaj > cx.betath || itgd - it_fb <= 1) { imeth = cx.gd_meth; kdown = cx.kdown; }
    else { imeth = 2; kdown = cx.kdowfb; it_fb = itgd; }
    double *dvx = dv.c[0].data(), *dvy = dv.c[1].data(), *vx = v.c[0].data(), *vy = v.c[1].data();
    const double *tx = t.c[0].data(), *ty = t.c[1].data();
    if (imeth == 1) {
        for (int iy = 1; iy <= my; iy++) {
            int ii = (mx - 1) + (iy - 1) * mx;
            vx[ii] = 0.0; vy[ii] = 0.0;
            for (int ix = mx - 1; ix >= 1; ix--) {
                ii = (ix - 1) + (iy - 1) * mx;
                if (igs.el[ii] == Adhes) { vx[ii] = vx[ii + 1] + dvx[ii]; vy[ii] = vy[ii + 1] + dvy[ii]; }
                else if (igs.el[ii] == Slip) {
                    double vt = tx[ii] * dvx[ii] + ty[ii] * dvy[ii];
                    vt = fsign(1.0, vt) * std::min(std::fabs(vt), fac_v * trcbnd[ii]);
                    vx[ii] = tx[ii] * vt; vy[ii] = ty[ii] * vt;
                    dvx[ii] = vx[ii] - vx[ii + 1]; dvy[ii] = vy[ii] - vy[ii + 1];
                } else {
                    vx[ii] = 0.0; vy[ii] = 0.0;
                    dvx[ii] = -vx[ii + 1]; dvy[ii] = -vy[ii + 1];
                }
            }
        }
    } else if (imeth == 2) {
        std::vector<double> dxi(mx + 1), dyi(mx + 1);
        for (int iy = 1; iy <= my; iy++) {
            int ii0 = (iy - 1) * mx;
            for (int ix = 1; ix <= mx; ix++) { dxi[ix] = dvx[ii0 + ix - 1]; dyi[ix] = dvy[ii0 + ix - 1]; }
            int ii = ii0 + mx - 1;
            vx[ii] = 0.0; vy[ii] = 0.0;
            for (int ix = mx - 1; ix >= 1; ix--) {
                ii = ii0 + ix - 1;
                if (igs.el[ii] == Adhes) {
                    if (ix + kdown <= mx) {
                        vx[ii] = vx[ii + 1] + dxi[ix] - dxi[ix + kdown];
                        vy[ii] = vy[ii + 1] + dyi[ix] - dyi[ix + kdown];
                    } else {
                        vx[ii] = vx[ii + 1] + dxi[ix];
                        vy[ii] = vy[ii + 1] + dyi[ix];
                    }
                    dvx[ii] = vx[ii] - vx[ii + 1]; dvy[ii] = vy[ii] - vy[ii + 1];
                } else if (igs.el[ii] == Slip) {
                    double vt = tx[ii] * dxi[ix] + ty[ii] * dyi[ix];
                    vt = fsign(1.0, vt) * std::min(std::fabs(vt), fac_v * trcbnd[ii]);
                    vx[ii] = tx[ii] * vt; vy[ii] = ty[ii] * vt;
                    dvx[ii] = vx[ii] - vx[ii + 1]; dvy[ii] = vy[ii] - vy[ii + 1];
                    for (int kk = 1; kk <= kdown; kk++) if (ix + kk <= mx) { dxi[ix + kk] = 0.0; dyi[ix + kk] = 0.0; }
                } else {
                    vx[ii] = 0.0; vy[ii] = 0.0;
                    dvx[ii] = -vx[ii + 1]; dvy[ii] = -vy[ii + 1];
                    for (int kk = 1; kk <= kdown; kk++) if (ix + kk <= mx) { dxi[ix + kk] = 0.0; dyi[ix + kk] = 0.0; }
                }
            }
        }
    } else if (imeth == 3) {
        for (int iy = 1; iy <= my; iy++) {
            int ii = (mx - 1) + (iy - 1) * mx;
            vx[ii] = 0.0; vy[ii] = 0.0;
            for (int ix = mx - 1; ix >= 1; ix--) {
                ii = (ix - 1) + (iy - 1) * mx;
                if (igs.el[ii] == Adhes) {
                    vx[ii] = cx.fdecay * vx[ii + 1] + dvx[ii]; vy[ii] = cx.fdecay * vy[ii + 1] + dvy[ii];
                    dvx[ii] = vx[ii] - vx[ii + 1]; dvy[ii] = vy[ii] - vy[ii + 1];
                } else if (igs.el[ii] == Slip) {
                    double vt = tx[ii] * dvx[ii] + ty[ii] * dvy[ii];
                    vt = fsign(1.0, vt) * std::min(std::fabs(vt), fac_v * trcbnd[ii]);
                    vx[ii] = tx[ii] * vt; vy[ii] = ty[ii] * vt;
                    dvx[ii] = vx[ii] - vx[ii + 1]; dvy[ii] = vy[ii] - vy[ii + 1];
                } else {
                    vx[ii] = 0.0; vy[ii] = 0.0;
                    dvx[ii] = -vx[ii + 1]; dvy[ii] = -vy[ii + 1];
                }
            }
        }
    }
}

// solve_elmtrc, gdsteady.f90:851-897
inline void solve_elmtrc(const Eldiv &igs, const std::vector<double> &mus, const double coefs[2][2], const GF3 &ps,
                         const GF3 &ss, Eldiv &igsopt, GF3 &psopt, GF3 &ssopt, int npot) {
    for (int ii = 0; ii < npot; ii++) {
        double pr[3] = {ps.c[0][ii], ps.c[1][ii], ps.c[2][ii]};
        double si[2] = {ss.c[0][ii], ss.c[1][ii]};
        int elnew = igs.el[ii];
        elmtrc(elnew, coefs, 1e-6, 1.0, 1.0, pr, mus[ii], si);
        igsopt.el[ii] = elnew;
        psopt.c[0][ii] = pr[0]; psopt.c[1][ii] = pr[1];
        ssopt.c[0][ii] = si[0]; ssopt.c[1][ii] = si[1];
    }
}

// compute_diagscaling, gdsteady.f90:901-1042.  'elnew' carries over between elements as in
// the reference; it starts at Exter.
inline void compute_diagscaling(const TangCtx &cx, const Eldiv &igs, const std::vector<double> &mus,
                                const double coefs[2][2], const GF3 &ps, const GF3 &ss, std::vector<double> &dscl) {
    const double tiny_err = 1e-6, epselm = 1e-6, omgscl = 1.0;
    const int mx = cx.mx, npot = cx.npot;
    int elnew = Exter;
    double fac_s = 0.0;
    for (int ii = 0; ii < npot; ii++) {
        if (igs.el[ii] == Slip) {
            double pr[3] = {ps.c[0][ii], ps.c[1][ii], ps.c[2][ii]};
            double si[2] = {ss.c[0][ii], ss.c[1][ii]};
            double th_p0 = std::atan2(pr[1], pr[0]);
            double th_s0 = std::atan2(-si[1], -si[0]);
            double err_0 = th_s0 - th_p0;
            if (std::fabs(err_0) >= pi) err_0 = err_0 - std::nearbyint(err_0 / (2.0 * pi)) * 2.0 * pi;
            if (std::fabs(err_0) <= tiny_err) {
                pr[0] = mus[ii] * pr[2] * std::cos(th_p0 + 0.1);
                pr[1] = mus[ii] * pr[2] * std::sin(th_p0 + 0.1);
                si[0] = ss.c[0][ii] + coefs[0][0] * (pr[0] - ps.c[0][ii]) + coefs[0][1] * (pr[1] - ps.c[1][ii]);
                si[1] = ss.c[1][ii] + coefs[1][0] * (pr[0] - ps.c[0][ii]) + coefs[1][1] * (pr[1] - ps.c[1][ii]);
                th_p0 = std::atan2(pr[1], pr[0]);
                th_s0 = std::atan2(-si[1], -si[0]);
                err_0 = th_s0 - th_p0;
                if (std::fabs(err_0) >= pi) err_0 = err_0 - std::nearbyint(err_0 / (2.0 * pi)) * 2.0 * pi;
            }
            if (std::fabs(err_0) > tiny_err) {
                elnew = igs.el[ii];
                elmtrc(elnew, coefs, epselm, 1.0, 1.0, pr, mus[ii], si);
                if (elnew == Slip) {
                    double th_p1 = std::atan2(pr[1], pr[0]);
                    double th_s1 = std::atan2(-si[1], -si[0]);
                    double upd_s = th_s1 - th_s0;
                    if (std::fabs(upd_s) >= pi) upd_s = upd_s - std::nearbyint(upd_s / (2.0 * pi)) * 2.0 * pi;
                    fac_s = std::fabs(upd_s) / std::fabs(err_0);
                }
            }
        }
        if (igs.el[ii] == Slip && elnew == Slip) {
            dscl[ii] = cx.d_slp * std::pow(fac_s, cx.pow_s);
        } else if (igs.el[ii] == Adhes || elnew == Adhes) {
            int ix = ii % mx + 1;
            int jx = ix;
            while (jx > 1 && igs.el[ii - ix + jx] == Adhes) jx--;
            double dscl_new;
            if (cx.d_cns < cx.d_ifc) dscl_new = std::max(cx.d_cns, cx.d_ifc + (ix - jx - 1) * std::min(0.0, cx.d_lin));
            else dscl_new = std::min(cx.d_cns, cx.d_ifc + (ix - jx - 1) * std::max(0.0, cx.d_lin));
            dscl[ii] = std::min(50.0 * dscl[ii], omgscl * dscl_new + (1.0 - omgscl) * dscl[ii]);
        } else {
            dscl[ii] = 0.0;
        }
    }
}

// perform_linesearch, gdsteady.f90:1046-1462.  Returns false when no bracket was found
// (the reference aborts the run there).
inline bool perform_linesearch(const TangCtx &cx, const Eldiv &igs, const std::vector<double> &trcbnd,
                               const std::vector<double> &dscl, const GF3 &dp, const GF3 &ss, const GF3 &dv,
                               const GF3 &v, const GF3 &q, const GF3 &told, double alpha0, double &alpha_j, int &j) {
    const int max_j = 99;
    const double tiny = 1e-12, eps_j = 0.001;
    const int mx = cx.mx, my = cx.my, npot = cx.npot;
    GF3 dpnew, psnew; dpnew.init(npot); psnew.init(npot);
    int tbl_j[max_j + 2];
    double tbl_alpha[max_j + 2], tbl_rho[max_j + 2], tbl_drhoda[max_j + 2];
    for (int k = 0; k < max_j + 2; k++) { tbl_j[k] = 0; tbl_alpha[k] = 0; tbl_rho[k] = 0; tbl_drhoda[k] = 0; }
    int itb_a = 0, itb_b = 0, itb_x = 0, itb_w = 0, itb_v = 0, itb_u = 0, ibrack = 1;
    double dst_cur = 0, dst_prv1 = 0, dst_prv2 = 0, ddrho = 0;
    j = 0; alpha_j = 0.0;
    double alpha_prv = -1.0;
    bool stop_j = false, has_bracket = false, prev_bracket;
    while (!stop_j) {
        double rhonew = 0, c0adh = 0, c1adh = 0, c0slp = 0, c1slp = 0, c2slp = 0;
        gf_copy(AllElm, dp, dpnew, ikTANG, igs);
        gf_axpy(AllInt, alpha_j, dv, dpnew, ikTANG, igs);
        apply_trcbnd(igs, trcbnd, dpnew, psnew, mx, my);
        for (int ii = 0; ii < npot; ii++) {
            double vt = v.c[0][ii] * told.c[0][ii] + v.c[1][ii] * told.c[1][ii];
            double tb = trcbnd[ii];
            double dth_da = (tb * vt) / (std::max(tiny, tb * tb) + alpha_j * alpha_j * vt * vt);
            double theta = std::atan2(psnew.c[1][ii], psnew.c[0][ii]);
            double nxn = std::cos(theta), nyn = std::sin(theta), txn = -nyn, tyn = nxn;
            double sx = ss.c[0][ii], sy = ss.c[1][ii], qx = q.c[0][ii], qy = q.c[1][ii];
            double sn = sx * nxn + sy * nyn;
            int elnew = igs.el[ii];
            if (elnew == Slip && sn > 0.0) elnew = Adhes;
            double st = sx * txn + sy * tyn, rt = -st;
            double qn = qx * nxn + qy * nyn, qt = qx * txn + qy * tyn;
            double d2 = dscl[ii] * dscl[ii];
            if (elnew == Adhes) {
                c0adh += 2.0 * d2 * (sx * qx + sy * qy);
                c1adh += 2.0 * d2 * (qx * qx + qy * qy);
                rhonew += d2 * ((sx + alpha_j * qx) * (sx + alpha_j * qx) + (sy + alpha_j * qy) * (sy + alpha_j * qy));
            } else if (elnew == Slip) {
                c0slp -= 2.0 * d2 * (rt * qt - rt * sn * dth_da);
                c1slp -= 2.0 * d2 * (-qt * qt + qt * sn * dth_da - rt * qn * dth_da);
                c2slp -= 2.0 * d2 * (qt * qn * dth_da);
                rhonew += d2 * (st + alpha_j * qt) * (st + alpha_j * qt);
            }
        }
        double drho_da = c0adh + c0slp + alpha_j * (c1adh + c1slp) + alpha_j * alpha_j * c2slp;
        // insert into table sorted on alpha (1-based positions)
        int itb = 1;
        while (itb <= j && alpha_j > tbl_alpha[itb]) itb++;
        itb_u = itb;
        for (int k = j; k >= itb; k--) {
            tbl_j[k + 1] = tbl_j[k]; tbl_alpha[k + 1] = tbl_alpha[k];
            tbl_rho[k + 1] = tbl_rho[k]; tbl_drhoda[k + 1] = tbl_drhoda[k];
        }
        if (has_bracket) {
            if (itb_a >= itb_u) itb_a++;
            if (itb_b >= itb_u) itb_b++;
            if (itb_x >= itb_u) itb_x++;
            if (itb_w >= itb_u) itb_w++;
            if (itb_v >= itb_u) itb_v++;
        }
        j++;
        tbl_j[itb] = j; tbl_alpha[itb] = alpha_j; tbl_rho[itb] = rhonew; tbl_drhoda[itb] = drho_da;
        prev_bracket = has_bracket;
        has_bracket = false;
        ibrack = 1;
        while (ibrack < j - 1 && !has_bracket) {
            has_bracket = (tbl_rho[ibrack + 1] <= std::min(tbl_rho[ibrack], tbl_rho[ibrack + 2]));
            if (!has_bracket) ibrack++;
        }
        if (has_bracket && !prev_bracket) {
            itb_a = ibrack; itb_x = ibrack + 1; itb_b = ibrack + 2;
            if (tbl_rho[itb_a] < tbl_rho[itb_b]) { itb_w = itb_a; itb_v = itb_b; }
            else { itb_w = itb_b; itb_v = itb_a; }
            dst_prv1 = tbl_alpha[itb_x] - tbl_alpha[itb_w];
            dst_prv2 = tbl_alpha[itb_w] - tbl_alpha[itb_v];
        } else if (has_bracket) {
            if (tbl_rho[itb_u] <= tbl_rho[itb_x]) {
                if (tbl_alpha[itb_u] >= tbl_alpha[itb_x]) itb_a = itb_x; else itb_b = itb_x;
                itb_v = itb_w; itb_w = itb_x; itb_x = itb_u;
            } else {
                if (tbl_alpha[itb_u] < tbl_alpha[itb_x]) itb_a = itb_u; else itb_b = itb_u;
                if (tbl_rho[itb_u] <= tbl_rho[itb_w] || tbl_alpha[itb_w] == tbl_alpha[itb_x]) {
                    itb_v = itb_w; itb_w = itb_u;
                } else if (tbl_rho[itb_u] <= tbl_rho[itb_v] || tbl_alpha[itb_v] == tbl_alpha[itb_x] ||
                           tbl_alpha[itb_v] == tbl_alpha[itb_w]) {
                    itb_v = itb_u;
                }
            }
            dst_prv2 = dst_prv1;
            dst_prv1 = dst_cur;
        }
        alpha_prv = alpha_j;
        if (has_bracket) {
            double xmid = 0.5 * (tbl_alpha[itb_a] + tbl_alpha[itb_b]);
            double tolx = eps_j * std::fabs(tbl_alpha[itb_x]) + tiny;
            bool ldone = (std::fabs(tbl_alpha[itb_x] - xmid) <= 2.0 * tolx - 0.5 * (tbl_alpha[itb_b] - tbl_alpha[itb_a]));
            if (!ldone) {
                bool use_parab;
                if (std::fabs(dst_prv2) <= tolx) {
                    use_parab = false;
                } else {
                    double br = (tbl_alpha[itb_x] - tbl_alpha[itb_w]) * (tbl_rho[itb_x] - tbl_rho[itb_v]);
                    double bq = (tbl_alpha[itb_x] - tbl_alpha[itb_v]) * (tbl_rho[itb_x] - tbl_rho[itb_w]);
                    double bp = (tbl_alpha[itb_x] - tbl_alpha[itb_v]) * bq - (tbl_alpha[itb_x] - tbl_alpha[itb_w]) * br;
                    bq = 2.0 * (bq - br);
                    if (bq > 0.0) bp = -bp;
                    bq = std::fabs(bq);
                    if (std::fabs(bp) >= std::fabs(0.5 * bq * dst_prv2) ||
                        bp <= bq * (tbl_alpha[itb_a] - tbl_alpha[itb_x]) ||
                        bp >= bq * (tbl_alpha[itb_b] - tbl_alpha[itb_x])) {
                        use_parab = false;
                    } else {
                        use_parab = true;
                        dst_cur = bp / bq;
                        alpha_j = tbl_alpha[itb_x] + dst_cur;
                        if (alpha_j - tbl_alpha[itb_a] < 2.0 * tolx || tbl_alpha[itb_b] - alpha_j < 2.0 * tolx)
                            dst_cur = tolx * fsign(1.0, xmid - tbl_alpha[itb_x]);
                    }
                }
                if (!use_parab) {
                    if (tbl_alpha[itb_x] >= xmid) dst_prv1 = tbl_alpha[itb_a] - tbl_alpha[itb_x];
                    else dst_prv1 = tbl_alpha[itb_b] - tbl_alpha[itb_x];
                    dst_cur = 0.381966 * dst_prv1;
                }
                alpha_j = tbl_alpha[itb_x] + dst_cur;
            }
        } else if (j == 1) {
            alpha_j = alpha_j + 0.6 * alpha0;
            ddrho = 10.0;
        } else if (tbl_rho[j] < tbl_rho[1]) {
            int ib = j - 1;
            double dal = tbl_alpha[ib + 1] - tbl_alpha[ib];
            if (j < 3) {
                ddrho = (tbl_drhoda[ib + 1] - tbl_drhoda[ib]) / dal;
                alpha_j = tbl_alpha[ib + 1] + std::min(3.0 * dal, -tbl_drhoda[ib] / ddrho);
            } else {
                alpha_j = tbl_alpha[ib + 1] + 3.0 * dal;
            }
        } else {
            int ib = 1;
            double dal = tbl_alpha[ib + 1] - tbl_alpha[ib];
            if (j < 3) {
                ddrho = (tbl_drhoda[ib + 1] - tbl_drhoda[ib]) / dal;
                alpha_j = tbl_alpha[ib] + std::min(-3.0 * dal, tbl_drhoda[ib] / ddrho);
            } else {
                alpha_j = tbl_alpha[ib] - 3.0 * dal;
            }
        }
        stop_j = (j >= max_j || std::fabs(alpha_j - alpha_prv) < eps_j * std::max(std::fabs(alpha_j), std::fabs(alpha_prv)));
    }
    if (!has_bracket) return false;
    if (j >= max_j) {
        int best = 1;
        for (int k = 2; k <= max_j; k++) if (tbl_rho[k] < tbl_rho[best]) best = k;
        alpha_j = tbl_alpha[best];
    }
    return true;
}

// gdsteady, gdsteady.f90:9-606 (elastic, no third-body layer).  Returns itgd (negative on
// stagnation like the reference); lstagn set as in the reference; 'bad' when the line search
// found no bracket.
inline int gdsteady(const TangCtx &cx, int maxgd, double eps, const GF3 &ws, Inflcf &cs, Eldiv &igs,
                    const std::vector<double> &mus, GF3 &ps, GF3 &ss, double &err, bool &lstagn, bool &bad) {
    const double tiny = 1e-12, fac_v = 1000.0;
    const int mx = cx.mx, my = cx.my, npot = cx.npot;
    bad = false;
    double coefs[2][2];
    const double flx = cs.use_3bl ? cs.flx_3bl : 0.0;     // gdsteady.f90:54-74
    coefs[0][0] = cs.ga_inv * cs.at(0, 0, 1, 1) + flx;
    coefs[0][1] = cs.ga_inv * cs.at(0, 0, 1, 2);
    coefs[1][0] = cs.ga_inv * cs.at(0, 0, 2, 1);
    coefs[1][1] = cs.ga_inv * cs.at(0, 0, 2, 2) + flx;
    Eldiv igsold = igs, igsopt = igs;
    GF3 dp, n, t, r, dv, v, q, psopt, ssopt, pold;
    for (GF3 *g : {&dp, &n, &t, &r, &dv, &v, &q, &psopt, &ssopt, &pold}) g->init(npot);
    std::vector<double> trcbnd(npot), dscl(npot), d_q0(npot), d_q1(npot);
    int nadh, nslip, nplast, nexter;
    eldiv_count(igs, nadh, nslip, nplast, nexter);
    double facnel = std::sqrt((double)(float)npot / (double)(float)(nadh + nslip + nplast));
    for (int ii = 0; ii < npot; ii++) trcbnd[ii] = mus[ii] * ps.c[2][ii];
    for (int ii = 0; ii < npot; ii++) dscl[ii] = 1.0;
    int itgd = 0, it_fb = -99, tot_j = 0, its_j = 0;
    double dif = 2.0, difid = 1.0, dif1 = 0.0, beta = 1.0, alpha = 0.0, alpha0 = 0.0, alpha1 = 0.0;
    bool lchanged = false;
    lstagn = false;
    auto set_nt = [&]() {
        for (int ii = 0; ii < npot; ii++) {
            double th = std::atan2(ps.c[1][ii], ps.c[0][ii]);
            n.c[2][ii] = th;
            n.c[0][ii] = std::cos(th); n.c[1][ii] = std::sin(th);
            t.c[0][ii] = -n.c[1][ii]; t.c[1][ii] = n.c[0][ii];
        }
    };
    auto set_r = [&]() {
        gf_set(AllElm, 0.0, r, ikTANG, igs);
        for (int ii = 0; ii < npot; ii++) {
            if (igs.el[ii] == Adhes) {
                r.c[0][ii] = -ss.c[0][ii] * dscl[ii];
                r.c[1][ii] = -ss.c[1][ii] * dscl[ii];
            } else if (igs.el[ii] == Slip) {
                double st = t.c[0][ii] * ss.c[0][ii] + t.c[1][ii] * ss.c[1][ii];
                r.c[0][ii] = -st * t.c[0][ii] * dscl[ii];
                r.c[1][ii] = -st * t.c[1][ii] * dscl[ii];
            }
        }
    };
    set_nt();
    compute_dp(ps, dp, mx, my);
    gf_set(AllElm, 0.0, ss, ikTANG, igs);
    vecaijpj(igs, AllInt, ss, ikTANG, dp, igs, ikTANG, cs, mx, my);
    gf_axpy(AllInt, 1.0, ws, ss, ikTANG, igs);
    compute_diagscaling(cx, igs, mus, coefs, ps, ss, dscl);
    set_r();
    {
        double mxabs = 0.0;
        for (int ii = 0; ii < npot; ii++) mxabs = std::max(mxabs, std::max(std::fabs(r.c[0][ii]), std::fabs(r.c[1][ii])));
        if (mxabs < tiny) dif = 0.0;
    }
    while ((lchanged || dif > difid) && itgd < maxgd) {
        itgd++;
        gf_copy(AllElm, r, dv, ikTANG, igs);
        project_searchdir(cx, igs, trcbnd, itgd, it_fb, beta, t, dv, v, fac_v);
        vecaijpj(igs, AllInt, q, ikTANG, dv, igs, ikTANG, cs, mx, my);
        if (itgd <= 1) {
            alpha0 = 0.0; alpha1 = 0.0;
            for (int ii = 0; ii < npot; ii++) {
                alpha0 += r.c[0][ii] * r.c[0][ii] + r.c[1][ii] * r.c[1][ii];
                alpha1 += (r.c[0][ii] * q.c[0][ii] + r.c[1][ii] * q.c[1][ii]) * dscl[ii];
            }
            alpha0 = alpha0 / alpha1;
        } else {
            alpha0 = 0.5 * (alpha0 + alpha);
        }
        if (!perform_linesearch(cx, igs, trcbnd, dscl, dp, ss, dv, v, q, t, alpha0, alpha, its_j)) {
            bad = true; err = dif; return itgd;
        }
        tot_j += its_j;
        double nq = 0.0, nr = 0.0;
        for (int ii = 0; ii < npot; ii++) {
            if (igs.el[ii] >= Adhes) {
                double a0 = dscl[ii] * q.c[0][ii], a1 = dscl[ii] * q.c[1][ii];
                nq += a0 * a0 + a1 * a1;
                nr += r.c[0][ii] * r.c[0][ii] + r.c[1][ii] * r.c[1][ii];
            }
        }
        beta = alpha * std::sqrt(nq) / std::sqrt(nr);
        lchanged = false;
        igsold.el = igs.el;
        gf_copy(AllElm, ps, pold, ikTANG, igs);
        gf_axpy(AllInt, alpha, dv, dp, ikTANG, igs);
        apply_trcbnd(igs, trcbnd, dp, ps, mx, my);
        set_nt();
        gf_set(AllElm, 0.0, ss, ikTANG, igs);
        vecaijpj(igs, AllInt, ss, ikTANG, dp, igs, ikTANG, cs, mx, my);
        gf_axpy(AllInt, 1.0, ws, ss, ikTANG, igs);
        solve_elmtrc(igs, mus, coefs, ps, ss, igsopt, psopt, ssopt, npot);
        for (int ii = 0; ii < npot; ii++)
            if (igs.el[ii] == Adhes) {
                double ptabs = std::sqrt(ps.c[0][ii] * ps.c[0][ii] + ps.c[1][ii] * ps.c[1][ii]);
                if (ptabs >= trcbnd[ii] - tiny) { igs.el[ii] = Slip; lchanged = true; }
            }
        for (int ii = 0; ii < npot; ii++)
            if (igsold.el[ii] == Slip) {
                double snrm = n.c[0][ii] * ss.c[0][ii] + n.c[1][ii] * ss.c[1][ii];
                double cosdth = (n.c[0][ii] * psopt.c[0][ii] + n.c[1][ii] * psopt.c[1][ii]) / trcbnd[ii];
                if ((snrm > 0.0 && (dscl[ii] >= 0.001 || igsopt.el[ii] == Adhes)) || cosdth <= -0.5) {
                    igs.el[ii] = Adhes; lchanged = true;
                }
            }
        compute_diagscaling(cx, igs, mus, coefs, ps, ss, dscl);
        set_r();
        gf_axpy(AllInt, -1.0, ps, pold, ikTANG, igs);
        double facdif;
        if (beta >= 0.1) facdif = 1.0;
        else if (beta >= 0.001) facdif = 0.1 / beta;
        else facdif = 100.0;
        dif = facnel * gf_rms(AllElm, pold, ikTANG, igs) * facdif;
        difid = eps * std::max(1e-6, facnel * gf_rms(AllElm, ps, ikTANG, igs));
        if (itgd == 1) dif1 = dif;
    }
    double resrms = gf_rms(AllInt, r, ikTANG, igs);
    double res_dp = resrms / std::max(coefs[0][0], coefs[1][1]);
    err = dif;
    double conv = 1.0;
    if (dif * dif1 > 0.0 && itgd > 1) conv = std::exp(std::log(dif / dif1) / (itgd - 1));
    if (lchanged && itgd >= maxgd) {
        lstagn = true;
    } else if (dif > difid && conv > 1.0 && itgd >= maxgd) {
        lstagn = true;
    } else if (conv < 1.0 - tiny && res_dp > 5.0 * difid / (1.0 - conv)) {
        itgd = -itgd;
        lstagn = true;
    }
    (void)tot_j;
    return itgd;
}

// ------------------------------------------------------------------------------------------
// TangCG, m_solvpt.f90:1841-2442 (elastic, no plasticity)
// ------------------------------------------------------------------------------------------
inline int tangcg(const TangCtx &cx, int maxcg, double eps, const GF3 &ws, Inflcf &cs, Inflcf &ms, Eldiv &igs,
                  const std::vector<double> &mu, GF3 &ps, GF3 &ss, double &err, bool &bad,
                  bool is_sens = false) {
    const int num_inn = 4;
    const double small = 1e-6;
    const int mx = cx.mx, my = cx.my, npot = cx.npot;
    bad = false;
    double ga = cs.ga;
    bool use_fftprec = true;
    // is_sens: tolerance relative to the change from the initial estimate (m_solvpt.f90:1908-1914)
    GF3 ps0, tmp;
    if (is_sens) { ps0 = ps; tmp.init(npot); }
    if (std::max(std::fabs(cs.at(0, 0, 1, 2)), std::fabs(cs.at(0, 0, 2, 1))) >
        (double)1e-8f * std::min(cs.at(0, 0, 1, 1), cs.at(0, 0, 2, 2))) { bad = true; return 0; }
    fft_makeprec(1, cs, 1, ms);
    fft_makeprec(2, cs, 2, ms);
    int nadh, nslip, nplast, nexter;
    eldiv_count(igs, nadh, nslip, nplast, nexter);
    double facnel = std::sqrt((double)(float)npot / (double)(float)(nadh + nslip + nplast));
    GF3 n, t, r, z, v, q, pold;
    for (GF3 *g : {&n, &t, &r, &z, &v, &q, &pold}) g->init(npot);
    std::vector<double> g(npot);
    for (int ii = 0; ii < npot; ii++) g[ii] = mu[ii] * ps.c[2][ii];
    int itcg = 0, it_inn = 0;
    double dif = 2.0, difid = 1.0, difinn = 0.0, dif1 = 0.0, alpha = 0.0, trsinn = 0.0;
    bool lchanged = false;
    auto set_nt = [&]() {
        for (int ii = 0; ii < npot; ii++) {
            n.c[2][ii] = std::atan2(ps.c[1][ii], ps.c[0][ii]);
            n.c[0][ii] = std::cos(n.c[2][ii]); n.c[1][ii] = std::sin(n.c[2][ii]);
            t.c[0][ii] = -n.c[1][ii]; t.c[1][ii] = n.c[0][ii];
        }
    };
    auto set_r = [&]() {
        gf_copy(AllElm, ss, r, ikTANG, igs);
        gf_scal(AllElm, -1.0, r, ikTANG, igs);
        for (int ii = 0; ii < npot; ii++)
            if (igs.el[ii] == Slip) {
                double perp = t.c[0][ii] * r.c[0][ii] + t.c[1][ii] * r.c[1][ii];
                r.c[0][ii] = perp * t.c[0][ii]; r.c[1][ii] = perp * t.c[1][ii];
            }
    };
    set_nt();
    gf_set(AllElm, 0.0, ss, ikTANG, igs);
    vecaijpj(igs, AllInt, ss, ikTANG, ps, igs, ikTANG, cs, mx, my);
    gf_axpy(AllInt, 1.0, ws, ss, ikTANG, igs);
    set_r();
    while ((lchanged || dif > difid) && itcg < maxcg) {
        itcg++; it_inn++;
        if (use_fftprec) {
            if (nslip + nplast > 3 * nadh && my > 1) use_fftprec = false;
            if (itcg >= maxcg / 2) use_fftprec = false;
            if (!use_fftprec) lchanged = true;
        }
        if (use_fftprec) {
            vecaijpj(igs, AllInt, z, ikX, r, igs, ikX, ms, mx, my);
            vecaijpj(igs, AllInt, z, ikY, r, igs, ikY, ms, mx, my);
        } else {
            gf_copy(AllElm, r, z, ikTANG, igs);
        }
        for (int ii = 0; ii < npot; ii++) {
            if (igs.el[ii] == Slip) {
                double snrm = -ss.c[0][ii] * n.c[0][ii] - ss.c[1][ii] * n.c[1][ii];
                z.c[0][ii] = z.c[0][ii] / (cs.at(0, 0, 1, 1) + ga * snrm / g[ii]);
                z.c[1][ii] = z.c[1][ii] / (cs.at(0, 0, 2, 2) + ga * snrm / g[ii]);
            } else {
                z.c[0][ii] = z.c[0][ii] / cs.at(0, 0, 1, 1);
                z.c[1][ii] = z.c[1][ii] / cs.at(0, 0, 2, 2);
            }
        }
        for (int ii = 0; ii < npot; ii++)
            if (igs.el[ii] == Slip) {
                double perp = t.c[0][ii] * z.c[0][ii] + t.c[1][ii] * z.c[1][ii];
                z.c[0][ii] = perp * t.c[0][ii]; z.c[1][ii] = perp * t.c[1][ii];
            }
        if (itcg <= 1 || lchanged) {
            gf_copy(AllElm, z, v, ikTANG, igs);
        } else {
            double zq = gf_dot(AllElm, z, q, ikTANG, igs);
            double vq = gf_dot(AllElm, v, q, ikTANG, igs);
            double beta;
            if (std::fabs(zq) < 1e-60 || std::fabs(vq) < small * std::fabs(zq)) beta = 0.0;
            else beta = -zq / vq;
            gf_scal(AllElm, beta, v, ikTANG, igs);
            gf_axpy(AllElm, 1.0, z, v, ikTANG, igs);
        }
        vecaijpj(igs, AllInt, q, ikTANG, v, igs, ikTANG, cs, mx, my);
        for (int ii = 0; ii < npot; ii++)
            if (igs.el[ii] == Slip) {
                double perp = t.c[0][ii] * q.c[0][ii] + t.c[1][ii] * q.c[1][ii];
                q.c[0][ii] = perp * t.c[0][ii]; q.c[1][ii] = perp * t.c[1][ii];
            }
        for (int ii = 0; ii < npot; ii++)
            if (igs.el[ii] == Slip) {
                double snrm = (n.c[0][ii] * ss.c[0][ii] + n.c[1][ii] * ss.c[1][ii]) / g[ii];
                q.c[0][ii] -= snrm * v.c[0][ii]; q.c[1][ii] -= snrm * v.c[1][ii];
            }
        double rv = gf_dot(AllElm, r, v, ikTANG, igs);
        double vq = gf_dot(AllElm, v, q, ikTANG, igs);
        if (std::fabs(rv) < 1e-60) alpha = 0.0;
        else if (std::fabs(vq) < small * std::fabs(rv)) alpha = 1.0;
        else alpha = rv / vq;
        gf_copy(AllElm, ps, pold, ikTANG, igs);
        gf_axpy(AllInt, alpha, v, ps, ikTANG, igs);
        for (int ii = 0; ii < npot; ii++)
            if (igs.el[ii] == Slip) {
                double ptabs = std::sqrt(ps.c[0][ii] * ps.c[0][ii] + ps.c[1][ii] * ps.c[1][ii]);
                ps.c[0][ii] = ps.c[0][ii] * g[ii] / ptabs;
                ps.c[1][ii] = ps.c[1][ii] * g[ii] / ptabs;
            }
        dif = alpha * facnel * gf_rms(AllElm, v, ikTANG, igs);
        difinn += dif;
        if (itcg <= 5 || itcg % 5 == 1) {
            double ptang;
            if (!is_sens) {
                ptang = facnel * gf_rms(AllElm, ps, ikTANG, igs);
            } else {
                gf_copy(AllElm, ps, tmp, ikTANG, igs);
                gf_axpy(AllElm, -1.0, ps0, tmp, ikTANG, igs);
                ptang = facnel * gf_rms(AllElm, tmp, ikTANG, igs);
            }
            difid = eps * std::max(1e-6, ptang);
            trsinn = (double)0.01f * ptang;
        }
        if (it_inn >= num_inn || dif <= difid || difinn > trsinn) {
            lchanged = false;
            for (int ii = 0; ii < npot; ii++)
                if (igs.el[ii] == Adhes) {
                    double ptabs = std::sqrt(ps.c[0][ii] * ps.c[0][ii] + ps.c[1][ii] * ps.c[1][ii]);
                    if (ptabs > g[ii]) {
                        igs.el[ii] = Slip;
                        ps.c[0][ii] = ps.c[0][ii] * g[ii] / ptabs;
                        ps.c[1][ii] = ps.c[1][ii] * g[ii] / ptabs;
                        lchanged = true;
                    }
                }
            vecaijpj(igs, AllInt, ss, ikTANG, ps, igs, ikTANG, cs, mx, my);
            gf_axpy(AllInt, 1.0, ws, ss, ikTANG, igs);
            for (int ii = 0; ii < npot; ii++)
                if (igs.el[ii] == Slip) {
                    double snrm = ss.c[0][ii] * ps.c[0][ii] + ss.c[1][ii] * ps.c[1][ii];
                    if (snrm > 0.0) { igs.el[ii] = Adhes; lchanged = true; }
                }
            gf_axpy(AllElm, -1.0, ps, pold, ikTANG, igs);
            dif = facnel * gf_rms(AllElm, pold, ikTANG, igs);
            it_inn = 0;
            difinn = 0.0;
            if (lchanged) eldiv_count(igs, nadh, nslip, nplast, nexter);
        }
        if (itcg == 1) dif1 = dif;
        if ((lchanged || dif > difid) && itcg < maxcg) {
            if (it_inn <= 0) { set_nt(); set_r(); }
            else gf_axpy(AllInt, -alpha, q, r, ikTANG, igs);
        }
    }
    err = dif;
    (void)dif1;
    return itcg;
}

} // namespace orc
