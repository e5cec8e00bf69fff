// CPU ORACLE -- test infrastructure only (see contact_oracle.h).
//
// Case driver: contac / panprc (m_scontc.f90:37-553), set-up (m_sdis.f90), influence
// coefficients (sgencr, m_visc.f90:127-376), TANG (m_stang.f90:28-951), output quantities
// (soutpt, m_soutpt.f90:377-511) and the cntc_calculate error mapping
// (contact_addon.f90:3870-3890).
#include "contact_oracle.h"
#include "orc_hertz.hpp"
#include "orc_norm.hpp"
#include "orc_tang.hpp"
#include "orc_subsurf.hpp"

using namespace orc;

namespace {

constexpr int CNTC_err_norm = -27, CNTC_err_tang = -28, CNTC_err_other = -99;

struct Case {
    const orc_problem *pb;
    // geometry
    int mx, my, npot;
    double dx, dy, dxdy, xl, yl, xc1, yc1;
    Grid g;
    // Hertz
    double a1 = 0, b1 = 0, aa = 0, bb = 0, aob = 0, rho = 0, cp = 0, scale = 1;
    // material
    double ga, nu, ak;
    // kinematics
    double chi, dq, veloc, pen, fntrue, cksi, ceta, cphi, muscal;
    // solver
    TangCtx tc;
    int maxout;
    // state
    Eldiv igs, igv;                 // current and previous element division
    GF3 ps, hs, us, ss, pv;         // pv: tractions of the previous time instance
    std::vector<double> mus;
    Inflcf cs, cv, ms;
    int itnorm = 0, ittang = 0, itcg = 0, itgs = 0, solver_eff = 0;
    bool unsupported = false, aborted = false;
    // sensitivities sens(iout, iin) (t_output%sens, m_hierarch_data.f90:122-128, 814):
    // iout 0..3 = Fn, Fx, Fy, Mz; iin 0..3 = pen, cksi, ceta, cphi
    double sens[4][4] = {};
    // Newton-Raphson history on the creepages: per iteration ittang, itnr, cksi, Fx/(mu Fn),
    // ceta, Fy/(mu Fn), solver iterations
    std::vector<double> nr_hist;
    // falling friction: the static coefficient of the law, the history of the slip loop
    double fstat_eff = 0.0;
    std::vector<double> slp_hist;
    std::vector<double> muv, svx, svy;   // previous coefficient of friction and shift (set_prev_data)
    // ConvexGS: contact elements, leading edge, and for steady rolling csv = cs - cv
    std::vector<int> iel, ii2j;
    Ledg ledg;
    Inflcf csv;
    bool have_csv = false;
};

constexpr int iout_fn = 0, iout_fx1 = 1, iout_fy1 = 2, iout_mz1 = 3;
constexpr int iin_dpen = 0, iin_dksi1 = 1, iin_deta1 = 2, iin_dphi1 = 3;

// set_tang_rhs, m_sdis.f90:498-583 (M=0, no extra rhs)
void set_tang_rhs(Case &c) {
    const orc_problem *pb = c.pb;
    bool is_roll = pb->tang == 2 || pb->tang == 3;
    double facphi = 1.0 / 6.0;
    double xofs = is_roll ? std::cos(c.chi) * c.dq * facphi : 0.0;
    double yofs = is_roll ? std::sin(c.chi) * c.dq * facphi : 0.0;
    for (int ii = 0; ii < c.npot; ii++) {
        c.hs.vx(ii) = 1.0 * -(c.g.y[ii] + yofs - 0.0) * c.cphi + 0.0;
        c.hs.vy(ii) = 1.0 * (c.g.x[ii] + xofs - 0.0) * c.cphi + 0.0;
    }
    if (pb->force3 == 0) for (int ii = 0; ii < c.npot; ii++) c.hs.vx(ii) += c.cksi;
    if (pb->force3 <= 1) for (int ii = 0; ii < c.npot; ii++) c.hs.vy(ii) += c.ceta;
    for (int ii = 0; ii < c.npot; ii++) { c.hs.vx(ii) *= -c.dq; c.hs.vy(ii) *= -c.dq; }
}

// eldiv0, m_sdis.f90:818-1009 (3-D case)
void eldiv0(Case &c) {
    const double facpen = (double)0.60f, reltol = (double)0.01f;
    const int maxit = 50;
    double fnscal = c.fntrue / c.ga;
    int imin = 0;
    for (int ii = 1; ii < c.npot; ii++) if (c.hs.vn(ii) < c.hs.vn(imin)) imin = ii;
    double hsmin = c.hs.vn(imin);
    double pentru = c.pen - hsmin;
    if (c.pb->norm == 1 && c.my == 1) {
        double rm = 1.0;
        double cdy = 0.35 - 0.05 * (std::log(c.dy) - std::log(200.0));
        pentru = std::pow(fnscal / c.dy * (1.0 - c.nu) / 0.6 / cdy / std::pow(rm, 0.1), (double)0.926f);
        c.pen = pentru + hsmin;
    } else if (c.pb->norm == 1) {
        double rmn = 1.0;
        double fac = rmn * 0.75 * std::sqrt(pi) * (1.0 - c.nu);
        double penmin = 0.0, fnmin = 0.0;
        double penmax = fac * fnscal / std::sqrt(c.dxdy);
        int ncnmax = 0;
        for (int ii = 0; ii < c.npot; ii++) if (c.hs.vn(ii) - hsmin < facpen * penmax) ncnmax++;
        double fnmax = penmax * std::sqrt(c.dxdy * ncnmax) / fac;
        int iter = 0;
        while (iter < maxit && std::fabs(fnmax - fnmin) > reltol * fnscal) {
            iter++;
            double penmid = 0.5 * (penmax + penmin);
            int ncnmid = 0;
            for (int ii = 0; ii < c.npot; ii++) if (c.hs.vn(ii) - hsmin < facpen * penmid) ncnmid++;
            double fnmid = penmid * std::sqrt(c.dxdy * ncnmid) / fac;
            if (fnmid < fnscal) { penmin = penmid; fnmin = fnmid; }
            else { penmax = penmid; fnmax = fnmid; }
        }
        pentru = penmax;
        c.pen = pentru + hsmin;
    }
    for (int ii = 0; ii < c.npot; ii++)
        c.igs.el[ii] = (c.hs.vn(ii) - hsmin < facpen * pentru) ? Adhes : Exter;
}

// init_curr_data, m_sdis.f90:587-770 (B=0,2,3; I=0..3)
void init_curr_data(Case &c, int ihertz) {
    const orc_problem *pb = c.pb;
    c.us.init(c.npot);
    if (pb->iestim == 0) for (int ii = 0; ii < c.npot; ii++) c.ps.vn(ii) = 0.0;
    if (pb->iestim == 0 || pb->iestim == 2 || pb->tang == 0)
        for (int ii = 0; ii < c.npot; ii++) { c.ps.vx(ii) = 0.0; c.ps.vy(ii) = 0.0; }
    bool use_hz = (pb->iestim == 0 && pb->bound == 0 && ihertz >= 1);
    if (pb->bound == 2 || use_hz) {
        if (ihertz <= 3) {
            double pnmax = 3.0 * c.fntrue / (2.0 * pi * c.aa * c.bb);
            for (int ii = 0; ii < c.npot; ii++) {
                double f = 1.0 - (c.g.x[ii] / c.aa) * (c.g.x[ii] / c.aa) - (c.g.y[ii] / c.bb) * (c.g.y[ii] / c.bb);
                c.ps.vn(ii) = pnmax * std::sqrt(std::max(0.0, f));
            }
        }
    }
    if (pb->bound == 3 && ihertz <= 3) {
        double pnmax = 2.0 * c.fntrue / (pi * c.aa * c.bb);
        for (int ii = 0; ii < c.npot; ii++) {
            double f = 1.0 - (c.g.x[ii] / c.aa) * (c.g.x[ii] / c.aa) - (c.g.y[ii] / c.bb) * (c.g.y[ii] / c.bb);
            c.ps.vn(ii) = pnmax * std::max(0.0, f);
        }
    }
    if ((pb->bound >= 2 && pb->bound <= 4) || use_hz) {
        for (int ii = 0; ii < c.npot; ii++) c.igs.el[ii] = (c.ps.vn(ii) > (double)1e-20f) ? Adhes : Exter;
    } else if (pb->iestim == 0) {
        eldiv0(c);
    }
    if (pb->iestim == 1) {
        for (int ii = 0; ii < c.npot; ii++) {
            if (c.igs.el[ii] <= Exter) { c.ps.vn(ii) = 0; c.ps.vx(ii) = 0; c.ps.vy(ii) = 0; }
            else if (c.igs.el[ii] == Slip) {
                double pabs = std::max(1e-10, std::sqrt(c.ps.vx(ii) * c.ps.vx(ii) + c.ps.vy(ii) * c.ps.vy(ii)));
                c.ps.vx(ii) = c.mus[ii] * c.ps.vn(ii) * c.ps.vx(ii) / pabs;
                c.ps.vy(ii) = c.mus[ii] * c.ps.vn(ii) * c.ps.vy(ii) / pabs;
            }
        }
    }
    if (pb->iestim == 2)
        for (int ii = 0; ii < c.npot; ii++) if (c.igs.el[ii] >= Adhes) c.igs.el[ii] = Adhes;
    for (int ii = 0; ii < c.npot; ii++) if (c.hs.vn(ii) > (double)1e29f) c.igs.el[ii] = Exter;
    areas(c.igs);
    // initial sensitivities and creepages, m_sdis.f90:754-766
    if (pb->iestim == 0) for (int io = iout_fx1; io <= iout_mz1; io++) c.sens[io][iin_dpen] = 0.0;
    if (pb->iestim == 0 && (pb->norm != 1 || ihertz != 0)) c.sens[iout_fn][iin_dpen] = 0.0;
    if (pb->iestim == 0 || pb->iestim == 2) {
        if (pb->force3 >= 1) c.cksi = 1e-6;
        if (pb->force3 == 2) c.ceta = 0.0;
        for (int io = iout_fn; io <= iout_mz1; io++)
            for (int ji = iin_dksi1; ji <= iin_dphi1; ji++) c.sens[io][ji] = 0.0;
    }
}

// stang_rhs, m_stang.f90:749-951: the fixed part of the shift, wsfix = -facdt h + u(ps_n)
// - u'(pv): for steady rolling u' of the current pressure through cv; for shifts and transient
// rolling u' of the previous tractions (normal and tangential), and at the leading edge of
// transient rolling the edge estimate ubnd of the previous tractions
void stang_rhs(Case &c, const std::vector<int> &iel, const std::vector<double> &facdt, GF3 &wsfix) {
    const int mx = c.mx, my = c.my, n = c.npot;
    const bool is_ssrol = c.pb->tang == 3;
    areas(c.igs);
    areas(c.igv);
    GF3 usn, uvn, uvt; usn.init(n); uvn.init(n); uvt.init(n);
    GF3 wsrig; wsrig.init(n);
    for (int ik = 1; ik <= 2; ik++)
        for (int ii : iel) wsrig.c[ik - 1][ii] = -facdt[ii] * c.hs.c[ik - 1][ii];
    vecaijpj(c.igs, AllInt, usn, ikTANG, c.ps, c.igs, ikZ, c.cs, mx, my);
    if (!is_ssrol) {
        vecaijpj(c.igs, AllInt, uvn, ikTANG, c.pv, c.igv, ikZ, c.cv, mx, my);
        vecaijpj(c.igs, AllInt, uvt, ikTANG, c.pv, c.igv, ikTANG, c.cv, mx, my);
    } else {
        vecaijpj(c.igs, AllInt, uvn, ikTANG, c.ps, c.igs, ikZ, c.cv, mx, my);
    }
    std::vector<double> ubnd;
    subnd(c.tc, c.ledg, c.pv, c.igv, c.cs, ubnd);
    for (int ik = 1; ik <= 2; ik++)
        for (int ii : iel) {
            const int j = c.ii2j[ii];
            double w;
            if (is_ssrol) w = wsrig.c[ik - 1][ii] + usn.c[ik - 1][ii] - uvn.c[ik - 1][ii];
            else if (j <= 0) w = wsrig.c[ik - 1][ii] + usn.c[ik - 1][ii] - uvn.c[ik - 1][ii] - uvt.c[ik - 1][ii];
            else w = wsrig.c[ik - 1][ii] + usn.c[ik - 1][ii] - ubnd[(size_t)2 * j + ik - 1];
            wsfix.c[ik - 1][ii] = w;
        }
}

// tang_solver, m_solvpt.f90:382-493; is_sens: the sensitivity solve (mxsens, epsens)
int tang_solver(Case &c, const GF3 &wstot, int &info1, double &err, bool is_sens = false) {
    TangCtx &tc = c.tc;
    int it = 0;
    bool bad = false;
    int maxit = is_sens ? c.pb->mxsens : tc.maxgs;
    double eps = is_sens ? c.pb->epsens : tc.eps;
    if (c.solver_eff == isolv_stdygs) {
        it = stdygs(tc, wstot, c.cs, c.igs, c.mus, c.ps, c.ss, eps, maxit, tc.omegah, tc.omegas, info1, err, bad,
                    is_sens);
    } else if (c.solver_eff == isolv_gdstdy) {
        bool lstagn = false;
        it = gdsteady(tc, maxit, eps, wstot, c.cs, c.igs, c.mus, c.ps, c.ss, err, lstagn, bad);
        if (!bad && lstagn)
            it = stdygs(tc, wstot, c.cs, c.igs, c.mus, c.ps, c.ss, eps, maxit, tc.omegah, tc.omegas, info1, err, bad,
                        is_sens);
    } else if (c.solver_eff == isolv_tangcg) {
        it = tangcg(tc, maxit, eps, wstot, c.cs, c.ms, c.igs, c.mus, c.ps, c.ss, err, bad, is_sens);
    } else if (c.solver_eff == isolv_cnvxgs) {
        it = cnvxgs(tc, wstot, c.cs, c.have_csv ? &c.csv : nullptr, c.ledg, c.ii2j, c.iel, c.igs, c.mus, c.ps, c.ss,
                    eps, maxit, tc.omegah, tc.omegas, info1, err, is_sens);
    } else {
        c.unsupported = true;
        return 0;
    }
    if (bad) c.aborted = true;
    return it;
}

// relative total forces Fx/(mu Fn), Fy/(mu Fn) of the current tractions
void rel_forces(const Case &c, double &fx, double &fy) {
    fx = c.dxdy * gf_sum(AllElm, c.ps, ikX, c.igs) / (c.muscal * c.fntrue);
    fy = c.dxdy * gf_sum(AllElm, c.ps, ikY, c.igs) / (c.muscal * c.fntrue);
}

// solvpt, m_solvpt.f90:51-378: one tangential solve for the current element division; when
// total forces are prescribed (F=1: Fx, F=2: Fx and Fy) a Newton-Raphson iteration on cksi
// (and ceta) around it, with the derivatives taken as secants of its own steps.
int solvpt(Case &c, int ittang, const std::vector<int> &iel, const std::vector<double> &facdt, const GF3 &wsfix,
           int &info1, double &err) {
    const orc_problem *pb = c.pb;
    const int npot = c.npot, f3 = pb->force3;
    const double dq = c.dq;
    int nadh, nslip, nplast, nexter;
    areas(c.igs);
    eldiv_count(c.igs, nadh, nslip, nplast, nexter);
    GF3 wstot; wstot.init(npot);
    gf_copy(AllElm, wsfix, wstot, ikTANG, c.igs);
    if (f3 >= 1) for (int ii : iel) wstot.vx(ii) += facdt[ii] * c.cksi * dq;
    if (f3 >= 2) for (int ii : iel) wstot.vy(ii) += facdt[ii] * c.ceta * dq;
    info1 = 0;
    int it = tang_solver(c, wstot, info1, err);
    if (c.unsupported || c.aborted) return it;
    double fxkp1, fykp1;
    rel_forces(c, fxkp1, fykp1);
    int itgs = it;
    eldiv_count(c.igs, nadh, nslip, nplast, nexter);
    auto record = [&](int itnr, int its) {
        double row[7] = {(double)ittang, (double)itnr, c.cksi, fxkp1, c.ceta, fykp1, (double)its};
        c.nr_hist.insert(c.nr_hist.end(), row, row + 7);
    };
    double (&sens)[4][4] = c.sens;
    if (f3 >= 1 && info1 <= 1) {
        int itnr = 0;
        record(itnr, it);
        double df = std::fabs(pb->fxrel - fxkp1);
        if (f3 >= 2) df += std::fabs(pb->fyrel - fykp1);
        while (df > c.tc.eps && itnr < pb->maxnr && info1 <= 1) {
            itnr++;
            double dfx = pb->fxrel - fxkp1, dfy = pb->fyrel - fykp1;
            double dcksi = 0.0, dceta = 0.0;
            if (f3 == 1) {
                dceta = 0.0;
                if (std::fabs(sens[iout_fx1][iin_dksi1]) > (double)1e-6f) dcksi = dfx / sens[iout_fx1][iin_dksi1];
                else dcksi = (double)0.00003f;
            } else {
                double det = sens[iout_fx1][iin_dksi1] * sens[iout_fy1][iin_deta1] -
                             sens[iout_fy1][iin_dksi1] * sens[iout_fx1][iin_deta1];
                if (det > c.tc.eps) {
                    dcksi = (sens[iout_fy1][iin_deta1] * dfx - sens[iout_fy1][iin_dksi1] * dfy) / det;
                    dceta = (-sens[iout_fx1][iin_deta1] * dfx + sens[iout_fx1][iin_dksi1] * dfy) / det;
                } else {
                    dcksi = 0.000003;
                    dceta = 0.000003;
                }
            }
            int ithalf[2] = {0, 0};
            for (int ifxy = 1; ifxy <= f3; ifxy++) {
                double fxk = fxkp1, fyk = fykp1;
                if (ifxy == 1) {
                    c.cksi += dcksi;
                    for (int ii : iel) wstot.vx(ii) += facdt[ii] * dcksi * dq;
                } else {
                    c.ceta += dceta;
                    for (int ii : iel) wstot.vy(ii) += facdt[ii] * dceta * dq;
                }
                it = tang_solver(c, wstot, info1, err);
                if (c.unsupported || c.aborted) return itgs + it;
                rel_forces(c, fxkp1, fykp1);
                itgs += it;
                ithalf[ifxy - 1] = it;
                eldiv_count(c.igs, nadh, nslip, nplast, nexter);
                double dfxk = fxkp1 - fxk, dfyk = fykp1 - fyk;
                double scl = c.muscal * c.fntrue / ((nadh + nslip + nplast) * c.dxdy);
                if (ifxy == 1) {
                    if (nadh > 0) {
                        double dpxavg = dfxk * scl;
                        if (sens[iout_fx1][iin_dksi1] == 0.0 || std::fabs(dpxavg) > 10.0 * err)
                            sens[iout_fx1][iin_dksi1] = dfxk / dcksi;
                        double dpyavg = dfyk * scl;
                        if (std::fabs(dpyavg) > 10.0 * err) sens[iout_fy1][iin_dksi1] = dfyk / dcksi;
                    } else if (std::fabs(sens[iout_fx1][iin_dksi1]) < (double)1e-6f) {
                        sens[iout_fx1][iin_dksi1] = fxkp1 / c.cksi;
                    }
                } else {
                    if (nadh > 0) {
                        double dpxavg = dfxk * scl;
                        if (std::fabs(dpxavg) > 10.0 * err) sens[iout_fx1][iin_deta1] = dfxk / dceta;
                        double dpyavg = dfyk * scl;
                        if (sens[iout_fy1][iin_deta1] == 0.0 || std::fabs(dpyavg) > 10.0 * err)
                            sens[iout_fy1][iin_deta1] = dfyk / dceta;
                    } else if (std::fabs(sens[iout_fy1][iin_deta1]) < (double)1e-6f) {
                        sens[iout_fy1][iin_deta1] = fykp1 / c.ceta;
                    }
                }
                df = std::fabs(pb->fxrel - fxkp1);
                if (f3 >= 2) df += std::fabs(pb->fyrel - fykp1);
            }
            record(itnr, ithalf[0] + ithalf[1]);
        }
        // the reference adds the Newton-Raphson residual to the error estimate with the element
        // code Slip (= 2) in the place of the number of slip elements (m_solvpt.f90:361)
        err += 2.0 * df * c.muscal * c.fntrue / ((nadh + Slip + nplast) * c.dxdy);
    } else {
        sens[iout_fx1][iin_dksi1] = 0.0; sens[iout_fy1][iin_dksi1] = 0.0;
        sens[iout_fx1][iin_deta1] = 0.0; sens[iout_fy1][iin_deta1] = 0.0;
    }
    return itgs;
}

// linrol, m_hertz.f90:1147-1247: Kalker's creepage coefficients C11, C22, C23 of the linear
// theory for an elliptic contact with semi-axes ratio a/b, from his table of Cij at
// nu = 0, 1/4, 1/2 (Kalker 1990, table E.3) with the asymptotes for g = min(a/b, b/a) < 0.1.
// The table holds single-precision constants, as the reference's data statement does.
void linrol(double nu, double aob, double &cxx, double &cyy, double &cyz) {
    static const float cij[2][10][3][3] = {      // [a<b | a>b][g row][C11, C22, C23][nu 0, 1/4, 1/2]
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
    int icase;
    double g;
    if (aob <= 1.0) { g = aob; icase = 0; } else { g = 1.0 / aob; icase = 1; }
    if (icase == 0 && g < 0.101) {
        cxx = pi * pi / 4.0 / (1.0 - nu);
        cyy = pi * pi / 4.0;
        cyz = pi * std::sqrt(g) / 3.0 / (1.0 - nu) * (1.0 + nu * (std::log(16.0 / g) - 5.0));
    } else if (icase == 1 && g < 0.101) {
        double al = std::log(16.0 / (g * g));
        cxx = 2.0 * pi / (al - 2.0 * nu) / g * (1.0 + (3.0 - std::log(4.0)) / (al - 2.0 * nu));
        cyy = 2.0 * pi / g * (1.0 + (1.0 - nu) * (3.0 - std::log(4.0)) / ((1.0 - nu) * al + 2.0 * nu)) /
              ((1.0 - nu) * al + 2.0 * nu);
        cyz = 2.0 * pi / 3.0 / std::pow(g, 1.5) / ((1.0 - nu) * al - 2.0 + 4.0 * nu);
    } else {
        int irow = (int)(10.0 * g - 0.005);            // 1-based row, truncated as an integer assignment
        double fac = 10.0 * g - (double)(float)irow;
        double cc[3];
        for (int ic = 0; ic < 3; ic++) {
            double cn[3];
            for (int in = 0; in < 3; in++)
                cn[in] = fac * (double)cij[icase][irow][ic][in] + (1.0 - fac) * (double)cij[icase][irow - 1][ic][in];
            cc[ic] = (nu - 0.25) * (nu - 0.50) * 8.0 / cn[0] - (nu - 0.50) * nu * 16.0 / cn[1] +
                     nu * (nu - 0.25) * 8.0 / cn[2];
        }
        cxx = 1.0 / cc[0]; cyy = 1.0 / cc[1]; cyz = 1.0 / cc[2];
    }
}

// char_creep, m_solvpt.f90:497-540: characteristic creepages from the linear theory, with the
// contact's effective radius from its area and its semi-axes from the element bounding box
void char_creep(Case &c, double &ch_ksi, double &ch_eta, double &ch_phi) {
    int nadh, nslip, nplast, nexter;
    eldiv_count(c.igs, nadh, nslip, nplast, nexter);
    int ncon = nadh + nslip + nplast;
    double rc = std::sqrt((double)(float)ncon * c.dx * c.dy / pi);
    areas(c.igs);
    double a = (double)(float)std::max(1, c.igs.ixmax - c.igs.ixmin + 1) * c.dx * 0.5;
    double b = (double)(float)std::max(1, c.igs.iymax - c.igs.iymin + 1) * c.dy * 0.5;
    double c11, c22, c23;
    linrol(c.nu, a / b, c11, c22, c23);
    ch_ksi = c.fstat_eff * c.fntrue / (rc * rc * c.ga * c11);
    ch_eta = c.fstat_eff * c.fntrue / (rc * rc * c.ga * c22);
    ch_phi = c.fstat_eff * c.fntrue / (rc * rc * rc * c.ga * c23);
}

// sens_tang, m_solvpt.f90:544-796: d(Fx, Fy, Mz) / d(cksi, ceta, cphi) by one extra solve per
// creepage, perturbed by 1e-4 of its characteristic size and started from the solution,
// which is restored afterwards
void sens_tang(Case &c, const std::vector<int> &iel, const std::vector<double> &facdt, const GF3 &wsfix) {
    const int npot = c.npot, f3 = c.pb->force3;
    double fxrel, fyrel;
    rel_forces(c, fxrel, fyrel);
    auto moment = [&]() {
        double dx_y = 0, dy_x = 0;
        for (int ii = 0; ii < npot; ii++) { dx_y += c.ps.vx(ii) * c.g.y[ii]; dy_x += c.ps.vy(ii) * c.g.x[ii]; }
        return c.dxdy * (-dx_y + dy_x);
    };
    double mztrue = moment();
    double ch[3];
    char_creep(c, ch[0], ch[1], ch[2]);
    GF3 wstot; wstot.init(npot);
    gf_copy(AllElm, wsfix, wstot, ikTANG, c.igs);
    if (f3 >= 1) for (int ii : iel) wstot.vx(ii) += facdt[ii] * c.cksi * c.dq;
    if (f3 >= 2) for (int ii : iel) wstot.vy(ii) += facdt[ii] * c.ceta * c.dq;
    for (int icrp = iin_dksi1; icrp <= iin_dphi1; icrp++) {
        GF3 wsloc = wstot;
        double dcrp = 0.0001 * ch[icrp - iin_dksi1];
        for (int ii : iel) {
            if (icrp == iin_dksi1) wsloc.vx(ii) += facdt[ii] * dcrp * c.dq;
            else if (icrp == iin_deta1) wsloc.vy(ii) += facdt[ii] * dcrp * c.dq;
            else {
                wsloc.vx(ii) -= facdt[ii] * dcrp * c.g.y[ii] * c.dq;
                wsloc.vy(ii) += facdt[ii] * dcrp * c.g.x[ii] * c.dq;
            }
        }
        Eldiv igs0 = c.igs;
        GF3 ps0 = c.ps, us0 = c.us, ss0 = c.ss;
        int info1 = 0; double err = 0.0;
        tang_solver(c, wsloc, info1, err, true);
        if (c.unsupported || c.aborted) return;
        double fxloc, fyloc;
        rel_forces(c, fxloc, fyloc);
        double mzloc = moment();
        c.sens[iout_fx1][icrp] = (fxloc - fxrel) / dcrp;
        c.sens[iout_fy1][icrp] = (fyloc - fyrel) / dcrp;
        c.sens[iout_mz1][icrp] = (mzloc - mztrue) / dcrp;
        c.igs = igs0; c.ps = ps0; c.us = us0; c.ss = ss0;
    }
}

// fric_veldep_mu_steady, m_friclaw.f90:397-449: the coefficient of friction at steady sliding
// with velocity v for the falling laws L = 2 (linear), 3 (rational), 4 (exponential)
double mu_steady(const orc_problem *pb, double v) {
    const double fkin = pb->flaw[0], f1 = pb->flaw[1], f2 = pb->flaw[3];
    // a term that is absent gets a velocity scale of at least 1e-4 (m_friclaw.f90:826-846)
    const double s1 = (f1 < 1e-8) ? std::max(1e-4, pb->flaw[2]) : pb->flaw[2];
    const double s2 = (f2 < 1e-8) ? std::max(1e-4, pb->flaw[4]) : pb->flaw[4];
    if (pb->frclaw == 2)
        return fkin + f1 * std::max(0.0, 1.0 - 0.5 * v / s1) + f2 * std::max(0.0, 1.0 - 0.5 * v / s2);
    if (pb->frclaw == 3) return fkin + f1 / (1.0 + v / s1) + f2 / (1.0 + (v / s2) * (v / s2));
    if (pb->frclaw == 4) return fkin + f1 * std::exp(-std::log(2.0) * v / s1) + f2 * std::exp(-std::log(2.0) * v / s2);
    return pb->fstat;
}

// stang, m_stang.f90:28-746 (Coulomb and falling friction)
int stang(Case &c) {
    const orc_problem *pb = c.pb;
    TangCtx &tc = c.tc;
    const int mx = c.mx, my = c.my, npot = c.npot;
    bool is_roll = pb->tang == 2 || pb->tang == 3, is_ssrol = pb->tang == 3;
    std::vector<int> iel;
    for (int ii = 0; ii < npot; ii++) if (c.igs.el[ii] >= Adhes) iel.push_back(ii);
    int k = (int)iel.size();
    int ixsta = (is_roll && std::fabs(c.chi - pi) < 0.01) ? mx : 1;
    int icount = 0;
    for (int iy = 1; iy <= my; iy++) if (c.igs.el[(ixsta - 1) + (iy - 1) * mx] >= Adhes) icount++;
    if (is_ssrol) {
        if (tc.gausei_eff == 5 && ixsta == 1) c.solver_eff = isolv_gdstdy;
        else if (tc.gausei_eff != 2) c.solver_eff = isolv_stdygs;
        else c.solver_eff = isolv_cnvxgs;
    } else {
        c.solver_eff = (tc.gausei_eff != 2) ? isolv_tangcg : isolv_cnvxgs;
    }
    if (icount > 0 && (c.solver_eff == isolv_stdygs || c.solver_eff == isolv_gdstdy)) c.solver_eff = isolv_cnvxgs;
    if (tc.gausei_eff == 0 || tc.gausei_eff == 4 || tc.gausei_eff == 5) {
        if (k <= 25) { tc.omegah = 1.0; tc.omegas = 1.0; }
        else if (is_ssrol && c.solver_eff == isolv_cnvxgs) { tc.omegah = 0.5; tc.omegas = 0.5; }
        else if (is_ssrol) {
            if (c.dx / c.dy <= 5.0) { tc.omegah = 0.9; tc.omegas = 1.0; }
            else if (c.dx / c.dy <= 15.0) { tc.omegah = 0.8; tc.omegas = 0.8; }
            else { tc.omegah = 0.8; tc.omegas = 0.6; }
        } else { tc.omegah = 0.5; tc.omegas = 0.5; }
    }
    std::vector<double> facdt;
    sxbnd(tc, c.solver_eff, c.igs, c.g, facdt, c.ii2j, &c.ledg);
    c.iel = iel;
    if (c.solver_eff == isolv_cnvxgs && is_ssrol && !c.have_csv) {
        // csv, m_visc.f90:289-354 (no dq scaling): the tangential rows of cs minus those of the
        // coefficients shifted by one rolling step; the normal row of cs
        Inflcf sh; sh.alloc(mx, my, c.dx, c.dy);
        elascf_pcwcns(c.ak, c.nu, mx, my, c.dx, c.dy, std::cos(c.chi) * c.dq, std::sin(c.chi) * c.dq, sh);
        c.csv.alloc(mx, my, c.dx, c.dy);
        c.csv.ga = c.ga; c.csv.ga_inv = 1.0 / c.ga; c.csv.nt_cpl = c.cs.nt_cpl;
        c.csv.use_3bl = c.cs.use_3bl; c.csv.flx_3bl = c.cs.flx_3bl;
        for (int jk = 0; jk < 3; jk++)
            for (size_t q = 0; q < c.cs.cf[0][0].size(); q++) {
                c.csv.cf[0][jk][q] = c.cs.cf[0][jk][q] - sh.cf[0][jk][q];
                c.csv.cf[1][jk][q] = c.cs.cf[1][jk][q] - sh.cf[1][jk][q];
                c.csv.cf[2][jk][q] = c.cs.cf[2][jk][q];
            }
        c.have_csv = true;
    }
    // falling friction: an outer iteration on the slip velocity, m_stang.f90:250-690; the
    // coefficient per element from the steady law at the last slip velocity, for steady
    // rolling carried from the leading edge with the friction memory
    const bool use_out_it = pb->frclaw >= 2 && pb->frclaw <= 4;
    const int ixinc = (is_roll && std::fabs(c.chi - pi) < 0.01) ? -1 : 1;
    const int ixend = (ixinc < 0) ? 1 : mx;
    const double dt = c.dq / std::max(1e-10, c.veloc);
    std::vector<double> slpvel(npot, 0.0), slpprv(npot, 0.0), musted(npot, 0.0), muv = c.muv;
    // initial slip velocity, m_stang.f90:250-264: the previous shift (INISLP 0), zero (> 0),
    // the rolling velocity (< 0)
    for (int ii = 0; ii < npot; ii++)
        slpvel[ii] = (pb->inislp == 0) ? std::sqrt(c.svx[ii] * c.svx[ii] + c.svy[ii] * c.svy[ii]) / dt
                   : (pb->inislp > 0) ? 0.0 : c.veloc;
    if (!use_out_it) c.mus.assign(npot, pb->fstat);
    double omgslp = pb->omgslp;
    int itslp = 0;
    bool zreasl = false;
    int ittang = 0, itgs = 0;
    bool zready = false;
    GF3 wsfix; wsfix.init(npot);
    GF3 tmp; tmp.init(npot);
    Eldiv igsprv;
    while (itslp <= std::max(1, tc.maxin - 10) && !zreasl) {
        itslp++;
        zreasl = true;
        slpprv = slpvel;
        igsprv = c.igs;
        if (use_out_it) {
            for (int ii = 0; ii < npot; ii++) musted[ii] = mu_steady(pb, slpvel[ii]);
            for (int iy = 1; iy <= my; iy++) {
                if (is_ssrol) muv[(ixend - 1) + (iy - 1) * mx] = c.fstat_eff;
                for (int ix = ixend; ; ix -= ixinc) {
                    const int ii = (ix - 1) + (iy - 1) * mx;
                    const double theta = (pb->memdst <= 1e-9) ? 0.0
                        : pb->memdst / (pb->memdst + dt * std::max(slpvel[ii], pb->mem_s0));
                    c.mus[ii] = theta * muv[ii] + (1.0 - theta) * musted[ii];
                    if (is_ssrol && ix != ixsta) muv[ii - ixinc] = c.mus[ii];
                    if (ix == ixsta) break;
                }
            }
        }
        stang_rhs(c, iel, facdt, wsfix);
        zready = false;
        while (!zready && ittang < tc.maxin) {
            ittang++;
            zready = true;
            int info = 0; double errpt = 0.0;
            int it = solvpt(c, ittang, iel, facdt, wsfix, info, errpt);
            if (c.unsupported || c.aborted) return -1;
            itgs += it;
            if (info >= 3) { zready = true; ittang = -1; }
            int newins = 0;
            double tol = std::sqrt(2.0) * errpt;
            for (int ii : iel) {
                if (c.igs.el[ii] == Adhes) {
                    double pabs = std::sqrt(c.ps.vx(ii) * c.ps.vx(ii) + c.ps.vy(ii) * c.ps.vy(ii));
                    if (pabs >= c.mus[ii] * c.ps.vn(ii) + tol) {
                        newins++;
                        c.igs.el[ii] = Slip;
                        c.ps.vx(ii) = c.ps.vx(ii) * c.mus[ii] * c.ps.vn(ii) / pabs;
                        c.ps.vy(ii) = c.ps.vy(ii) * c.mus[ii] * c.ps.vn(ii) / pabs;
                    }
                }
            }
            if (newins != 0) zready = false;
            if (zready) {
                areas(c.igs);
                int ii0 = (std::max(1, mx / 2) - 1) + (std::max(1, my / 2) - 1) * mx;
                gf_set(AllElm, 1.0, tmp, ikTANG, c.igs);
                double tol1 = errpt * 2.0 * std::fabs(aijpj(ii0, ikX, tmp, c.igs, ikX, c.cs, mx, my));
                double tol2 = errpt * 2.0 * std::fabs(aijpj(ii0, ikY, tmp, c.igs, ikY, c.cs, mx, my));
                int newadh = 0;
                for (int ii : iel) {
                    if (c.igs.el[ii] == Slip) {
                        double ww = c.ss.vx(ii) * c.ps.vx(ii) + c.ss.vy(ii) * c.ps.vy(ii);
                        double tl = tol1 * std::fabs(c.ps.vx(ii)) + tol2 * std::fabs(c.ps.vy(ii)) +
                                    errpt * (std::fabs(c.ss.vx(ii)) + std::fabs(c.ss.vy(ii)));
                        if (ww > tl) { c.igs.el[ii] = Adhes; newadh++; }
                    }
                }
                if (newadh != 0) zready = false;
                if (info > 0) zready = true;
            }
        }
        if (!zready) ittang = -1;
        if (use_out_it) {
            int nadh, nslip, nplast, nexter;
            eldiv_count(c.igs, nadh, nslip, nplast, nexter);
            int nchanged = 0;
            for (int ii = 0; ii < npot; ii++) if (c.igs.el[ii] != igsprv.el[ii]) nchanged++;
            for (int ii = 0; ii < npot; ii++)
                slpvel[ii] = (c.igs.el[ii] == Exter) ? 0.0
                    : std::sqrt(c.ss.vx(ii) * c.ss.vx(ii) + c.ss.vy(ii) * c.ss.vy(ii)) / dt;
            GF3 d, v; d.init(npot); v.init(npot);
            for (int ii = 0; ii < npot; ii++) { slpprv[ii] -= slpvel[ii]; d.vx(ii) = slpprv[ii]; v.vx(ii) = slpvel[ii]; }
            const double dif = gf_rms(AllInt, d, ikX, c.igs);
            const double difid = 0.001 * gf_rms(AllInt, v, ikX, c.igs);
            if (itslp > 1)
                for (int ii = 0; ii < npot; ii++)
                    if (c.igs.el[ii] == Slip && c.mus[ii] > muv[ii])
                        slpvel[ii] = std::max(0.0, slpvel[ii] - (omgslp - 1.0) * slpprv[ii]);
            double row[4] = {(double)nadh, (double)nslip, dif, difid};
            c.slp_hist.insert(c.slp_hist.end(), row, row + 4);
            if (dif > difid && nslip > 0) zreasl = false;
            if (!zreasl && nchanged > 0 && itslp % 20 == 0) omgslp = 0.8 * omgslp;
        }
    }
    c.itgs = itgs;
    if (pb->sens >= 3) {
        sens_tang(c, iel, facdt, wsfix);
        if (c.unsupported || c.aborted) return -1;
    }
    return ittang;
}

// soutpt, m_soutpt.f90:377-511 (force, moment, elastic energy, maximum pressure)
void soutpt(Case &c, orc_result *r) {
    const int mx = c.mx, my = c.my, npot = c.npot;
    areas(c.igs);
    vecaijpj(c.igs, AllInt, c.us, ikZ, c.ps, c.igs, -3, c.cs, mx, my);
    vecaijpj(c.igs, AllInt, c.us, ikTANG, c.ps, c.igs, -3, c.cs, mx, my);
    int nadh, nslip, nplast, nexter;
    eldiv_count(c.igs, nadh, nslip, nplast, nexter);
    if (c.pb->norm == 0) c.fntrue = c.dxdy * gf_sum(AllElm, c.ps, ikZ, c.igs);
    // prescribed total forces are reported as prescribed (m_soutpt.f90:427-434)
    double fxrel = (c.pb->force3 >= 1) ? c.pb->fxrel
                                       : c.dxdy * gf_sum(AllElm, c.ps, ikX, c.igs) / (c.fntrue * c.muscal + tiny_);
    double fyrel = (c.pb->force3 >= 2) ? c.pb->fyrel
                                       : c.dxdy * gf_sum(AllElm, c.ps, ikY, c.igs) / (c.fntrue * c.muscal + tiny_);
    double fxtrue = fxrel * (c.fntrue * c.muscal + tiny_);
    double fytrue = fyrel * (c.fntrue * c.muscal + tiny_);
    double dx_y = 0, dy_x = 0;
    for (int ii = 0; ii < npot; ii++) { dx_y += c.ps.vx(ii) * c.g.y[ii]; dy_x += c.ps.vy(ii) * c.g.x[ii]; }
    double mztrue = -c.dxdy * dx_y + c.dxdy * dy_x;
    if (std::fabs(mztrue) < 0.5 * c.tc.eps * (c.muscal * c.fntrue + tiny_)) mztrue = 0.0;
    // B=2..4 (normal problem skipped): no elastic energy, deformed distance zero (m_soutpt.f90:453-470)
    bool skipped = c.pb->bound >= 2 && c.pb->bound <= 4;
    double elen = skipped ? 0.0 : 0.5 * 1e-3 * c.dxdy * gf_dot(AllInt, c.us, c.ps, ikALL, c.igs);
    double pmax = gf_max(AllElm, c.ps, ikZ, c.igs);
    r->fn = c.fntrue; r->fx = fxtrue; r->fy = fytrue; r->mz = mztrue;
    r->elen = elen; r->pmax = pmax;
    r->ncon = nadh + nslip + nplast; r->nadh = nadh; r->nslip = nslip;
    for (int ii = 0; ii < npot; ii++) {
        c.ss.vn(ii) = skipped ? 0.0 : -c.pen + c.hs.vn(ii) + c.us.vn(ii);
        if (c.igs.el[ii] != Slip) { c.ss.vx(ii) = 0.0; c.ss.vy(ii) = 0.0; }
    }
}

} // namespace

extern "C" {

void orc_default_problem(orc_problem *pb) {
    std::memset(pb, 0, sizeof(*pb));
    pb->pvtime = 2; pb->bound = 0; pb->tang = 3; pb->norm = 1; pb->force3 = 0; pb->iestim = 0; pb->gausei = 0;
    pb->maxgs = 999; pb->maxin = 20; pb->maxnr = 25; pb->maxout = 1; pb->eps = 1e-5;   // solv_init
    pb->omegah = 0.9; pb->omegas = 1.0; pb->inislp = 0; pb->omgslp = 0.5;
    pb->kdowfb = 1; pb->fdecay = 0.9; pb->betath = 0.1;
    pb->d_ifc = 1.0; pb->d_lin = 1.0; pb->d_cns = 1.0; pb->d_slp = 1.0; pb->pow_s = 0.9;
    pb->poiss1 = 0.28; pb->poiss2 = 0.28; pb->gg1 = 1.0; pb->gg2 = 1.0;
    pb->fstat = 0.3; pb->fkin = 0.3;
    pb->veloc = 1e3; pb->chi = 0.0; pb->dq = -1.0;
    pb->ipotcn = -3; pb->ibase = 1;
    pb->sens = 1; pb->mxsens = 30; pb->epsens = 1e-4;                                   // solv_init
}

int orc_opt_fft_size(int n) { return opt_fft_size(n); }

double orc_eli(double elmodk, double *ellk, double *elle) { return eli(elmodk, *ellk, *elle); }

static void subs_store(const SubsPoint &r, double *o) {
    for (int i = 0; i < 3; i++) o[i] = r.u[i];
    o[3] = r.sighyd; o[4] = r.sigvm; o[5] = r.sigtr;
    for (int i = 0; i < 3; i++) o[6 + i] = r.sigmaj[i];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) o[9 + 3 * i + j] = r.sig[i][j];
}

void orc_subsurf_points(int mx, int my, double dx, double dy, double xc1, double yc1, const double *pn,
                        const double *px, const double *py, const double *gg, const double *poiss, int npts,
                        const double *xyz, double *out) {
    SubsLoad L{mx, my, dx, dy, xc1, yc1, pn, px, py, {gg[0], gg[1]}, {poiss[0], poiss[1]}};
    for (int q = 0; q < npts; q++) subs_store(sstres_point(L, xyz + 3 * q), out + (size_t)q * ORC_SUBS_NCOL);
}

void orc_subsurf_depths(int mx, int my, double dx, double dy, double xc1, double yc1, const double *pn,
                        const double *px, const double *py, const double *gg, const double *poiss, int nz,
                        const double *z, double *out) {
    SubsLoad L{mx, my, dx, dy, xc1, yc1, pn, px, py, {gg[0], gg[1]}, {poiss[0], poiss[1]}};
    std::vector<SubsPoint> r((size_t)mx * my);
    for (int iz = 0; iz < nz; iz++) {
        sstres_fft_depth(L, z[iz], r.data());
        for (size_t ii = 0; ii < r.size(); ii++) subs_store(r[ii], out + ((size_t)iz * r.size() + ii) * ORC_SUBS_NCOL);
    }
}

void orc_influence_coefficients(int mx, int my, double dx, double dy, double nu, double ak, double xshft,
                                double yshft, double *out) {
    Inflcf c; c.alloc(mx, my, dx, dy);
    elascf_pcwcns(ak, nu, mx, my, dx, dy, xshft, yshft, c);
    size_t blk = (size_t)4 * mx * my;
    for (int ik = 1; ik <= 3; ik++)
        for (int jk = 1; jk <= 3; jk++)
            std::memcpy(out + ((ik - 1) * 3 + (jk - 1)) * blk, c.cf[ik - 1][jk - 1].data(), blk * sizeof(double));
}

static void load_block(Inflcf &c, int mx, int my, const double *blk, double ga) {
    c.alloc(mx, my, 1.0, 1.0);
    std::memcpy(c.cf[2][2].data(), blk, (size_t)4 * mx * my * sizeof(double));
    c.ga = ga; c.ga_inv = 1.0 / ga;
}

void orc_convolve(int mx, int my, const double *cf_block, double ga, const double *p, double *u) {
    Inflcf c; load_block(c, mx, my, cf_block, ga);
    Eldiv e; e.init(mx, my); for (int &v : e.el) v = Adhes; areas(e);
    GF3 pp, uu; pp.init(mx * my); uu.init(mx * my);
    std::memcpy(pp.c[2].data(), p, sizeof(double) * mx * my);
    vecaijpj(e, AllElm, uu, ikZ, pp, e, ikZ, c, mx, my);
    std::memcpy(u, uu.c[2].data(), sizeof(double) * mx * my);
}

void orc_convolve_direct(int mx, int my, const double *cf_block, double ga, const double *p, double *u) {
    Inflcf c; load_block(c, mx, my, cf_block, ga);
    Eldiv e; e.init(mx, my); for (int &v : e.el) v = Adhes; areas(e);
    GF3 pp; pp.init(mx * my);
    std::memcpy(pp.c[2].data(), p, sizeof(double) * mx * my);
    for (int ii = 0; ii < mx * my; ii++) u[ii] = aijpj(ii, ikZ, pp, e, ikZ, c, mx, my);
}

int orc_calculate(const orc_problem *pb, orc_result *r) {
    Case c;
    c.pb = pb;
    r->ierror = 0;
    r->nout = 0;
    // combin_mater, m_hierarch_data.f90:1543-1553
    double gg1 = pb->gg1, gg2 = pb->gg2, p1 = pb->poiss1, p2 = pb->poiss2;
    c.ga = 2.0 / (1.0 / gg1 + 1.0 / gg2);
    c.nu = c.ga * (p1 / gg1 + p2 / gg2) / 2.0;
    c.ak = (c.ga / 4.0) * ((1.0 - 2.0 * p1) / gg1 - (1.0 - 2.0 * p2) / gg2);
    // M=0 elastic, M=4 with an elastic interfacial layer; a plastic layer (use_plast,
    // m_stang.f90:68) is not restated
    if ((pb->mater != 0 && pb->mater != 4) ||
        (pb->mater == 4 && (pb->tau_c0 > 1e-10 && pb->tau_c0 <= 1e10))) {
        r->ierror = CNTC_err_other; return r->ierror;
    }
    const bool use_3bl = pb->mater == 4 && pb->laythk >= 1e-10;           // inflcf_mater
    const double flx_3bl = pb->mater == 4 ? pb->laythk / pb->gg3 : 0.0;  // m_sinput.f90:955
    c.maxout = pb->maxout;
    if (c.maxout >= 2 && std::fabs(c.ak) < 1e-4) c.maxout = 1;
    if (c.maxout <= 1 && std::fabs(c.ak) >= 1e-4 && !pb->standalone) c.maxout = 10;
    c.fntrue = pb->fn; c.pen = pb->pen;
    c.cksi = pb->cksi; c.ceta = pb->ceta; c.cphi = pb->cphi;
    c.chi = pb->chi; c.veloc = pb->veloc;
    // the static coefficient of a falling law, fric_update (m_friclaw.f90:296-310)
    c.fstat_eff = (pb->frclaw >= 2 && pb->frclaw <= 4) ? pb->flaw[0] + pb->flaw[1] + pb->flaw[3] : pb->fstat;
    c.muscal = c.fstat_eff;
    // Hertzian solution & potential contact (hzsol m_hertz.f90:29-93, potcon_hertz)
    int ihertz = 0;
    c.mx = std::max(1, (int)std::nearbyint(pb->potprm[0]));
    c.my = std::max(1, (int)std::nearbyint(pb->potprm[1]));
    double xl, yl, xh, yh, dx, dy;
    if (pb->ipotcn <= -1 && pb->ipotcn >= -3) {
        const double epshz = (double)1e-9f;
        double e_star = c.ga / (1.0 - c.nu);
        c.scale = pb->potprm[4];
        if (pb->ipotcn == -3) { c.aa = pb->potprm[2]; c.bb = pb->potprm[3]; }
        else if (pb->ipotcn == -1) { c.a1 = pb->potprm[2]; c.b1 = pb->potprm[3]; }
        else { c.a1 = pb->potprm[2]; c.aob = pb->potprm[3]; }
        if (pb->ipotcn == -2)
            elliptic_to_curv(pb->norm, c.a1, c.aa, c.aob, c.b1, c.bb, c.cp, c.rho, c.fntrue, c.pen, e_star, epshz);
        else
            hzcalc3d(e_star, epshz, pb->ipotcn, c.a1, c.b1, c.aa, c.bb, pb->norm, c.pen, c.fntrue, c.cp, c.rho);
        if (pb->ipotcn != -2) c.aob = (c.aa <= tiny_ && c.bb <= tiny_) ? 1.0 : c.aa / c.bb;
        xl = -c.scale * std::max(1e-9, c.aa);
        yl = -c.scale * std::max(1e-9, c.bb);
        xh = -xl; yh = -yl;
        dx = (xh - xl) / c.mx; dy = (yh - yl) / c.my;
        ihertz = -pb->ipotcn;
    } else if (pb->ipotcn >= 1 && pb->ipotcn <= 4) {
        // potcon_fill, m_hierarch_data.f90:1801-1861
        double a = pb->potprm[2], b = pb->potprm[3], cc = pb->potprm[4], d = pb->potprm[5];
        if (pb->ipotcn == 1) { xl = a; yl = b; dx = cc; dy = d; }
        else if (pb->ipotcn == 2) { xl = a; yl = b; dx = (cc - a) / c.mx; dy = (d - b) / c.my; }
        else if (pb->ipotcn == 3) { dx = cc; dy = d; xl = a - 0.5 * dx; yl = b - 0.5 * dy; }
        else { dx = (cc - a) / std::max(1, c.mx - 1); dy = (d - b) / std::max(1, c.my - 1); xl = a - 0.5 * dx; yl = b - 0.5 * dy; }
    } else {
        r->ierror = CNTC_err_other; return r->ierror;
    }
    c.dx = dx; c.dy = dy; c.dxdy = dx * dy; c.xl = xl; c.yl = yl;
    c.xc1 = xl + 0.5 * dx; c.yc1 = yl + 0.5 * dy;
    c.npot = c.mx * c.my;
    c.g.create(c.mx, c.xc1, dx, c.my, c.yc1, dy);
    // check_roll_stepsize, m_sdis.f90:125-206
    bool is_roll = pb->tang == 2 || pb->tang == 3, is_ssrol = pb->tang == 3;
    c.dq = (pb->dq > 0.0) ? pb->dq : dx;
    if ((is_ssrol && pb->gausei != 2) || pb->mater == 4) {
        if (pb->tang >= 1 && std::fabs(c.chi) > 0.01 && std::fabs(c.chi - pi) > 0.01) c.chi = 0.0;
        c.dq = dx;
    }
    if (!is_roll) { c.chi = 0.0; c.dq = 1.0; c.veloc = 1.0; }
    // influence coefficients, sgencr m_visc.f90:127-376
    c.cs.alloc(c.mx, c.my, dx, dy); c.ms.alloc(c.mx, c.my, dx, dy);
    for (Inflcf *f : {&c.cs, &c.ms}) {
        f->ga = c.ga; f->ga_inv = 1.0 / c.ga; f->use_3bl = use_3bl; f->flx_3bl = flx_3bl;
    }
    elascf_pcwcns(c.ak, c.nu, c.mx, c.my, dx, dy, 0.0, 0.0, c.cs);
    bool nt_cpl = std::fabs(c.ak) >= 1e-6;
    c.cs.nt_cpl = nt_cpl; c.ms.nt_cpl = nt_cpl;
    if (is_roll && (nt_cpl || pb->tang == 2)) {
        c.cv.alloc(c.mx, c.my, dx, dy); c.cv.ga = c.ga; c.cv.ga_inv = 1.0 / c.ga; c.cv.nt_cpl = nt_cpl;
        c.cv.use_3bl = use_3bl; c.cv.flx_3bl = flx_3bl;
        elascf_pcwcns(c.ak, c.nu, c.mx, c.my, dx, dy, std::cos(c.chi) * c.dq, std::sin(c.chi) * c.dq, c.cv);
        for (int jk = 1; jk <= 3; jk++)
            for (size_t q = 0; q < c.cv.cf[0][0].size(); q++) {
                c.cv.cf[2][jk - 1][q] = c.cs.cf[2][jk - 1][q];
                double s1 = c.cs.cf[0][jk - 1][q] - c.cv.cf[0][jk - 1][q];
                double s2 = c.cs.cf[1][jk - 1][q] - c.cv.cf[1][jk - 1][q];
                c.cv.cf[0][jk - 1][q] = c.cs.cf[0][jk - 1][q] - s1;
                c.cv.cf[1][jk - 1][q] = c.cs.cf[1][jk - 1][q] - s2;
            }
    } else {
        c.cv = c.cs;
    }
    // undeformed distance, set_norm_rhs m_sdis.f90:321-494
    c.hs.init(c.npot);
    int ibase = (ihertz >= 1) ? 1 : pb->ibase;
    if (ibase == 1) {
        double prm[6] = {0, 0, 0, 0, 0, 0};
        if (ihertz >= 1) { prm[0] = c.a1; prm[2] = c.b1; }
        else for (int k = 0; k < 6 && k < pb->nprmudf; k++) prm[k] = pb->prmudf[k];
        for (int ii = 0; ii < c.npot; ii++) {
            double x = c.g.x[ii], y = c.g.y[ii];
            c.hs.vn(ii) = prm[0] * x * x + prm[1] * x * y + prm[2] * y * y + prm[3] * x + prm[4] * y + prm[5];
        }
    } else if (ibase == 9) {
        if (pb->nprmudf != c.npot || !pb->prmudf) { r->ierror = CNTC_err_other; return r->ierror; }
        for (int ii = 0; ii < c.npot; ii++) c.hs.vn(ii) = pb->prmudf[ii];
    } else {
        r->ierror = CNTC_err_other; return r->ierror;
    }
    set_tang_rhs(c);
    // initial estimate
    c.ps.init(c.npot);
    c.ss.init(c.npot);
    c.igs.init(c.mx, c.my);
    c.mus.assign(c.npot, c.fstat_eff);
    if (pb->iestim != 0 && pb->igs_init) {
        for (int ii = 0; ii < c.npot; ii++) {
            c.igs.el[ii] = pb->igs_init[ii];
            c.ps.vn(ii) = pb->pn_init ? pb->pn_init[ii] : 0.0;
            c.ps.vx(ii) = pb->px_init ? pb->px_init[ii] : 0.0;
            c.ps.vy(ii) = pb->py_init ? pb->py_init[ii] : 0.0;
        }
    }
    if (pb->sens_init)
        for (int io = 0; io < 4; io++)
            for (int ji = 0; ji < 4; ji++) c.sens[io][ji] = pb->sens_init[io + 4 * ji];
    // set_prev_data, m_sdis.f90:208-312: the previous time instance (P=0 all of it, P=1 the
    // normal part, P=2 none)
    c.pv.init(c.npot);
    c.igv.init(c.mx, c.my);
    if (pb->pvtime <= 1 && pb->igv_init) {
        for (int ii = 0; ii < c.npot; ii++) {
            c.igv.el[ii] = pb->igv_init[ii];
            c.pv.vn(ii) = pb->pvn_init ? pb->pvn_init[ii] : 0.0;
            if (pb->pvtime == 0) {
                c.pv.vx(ii) = pb->pvx_init ? pb->pvx_init[ii] : 0.0;
                c.pv.vy(ii) = pb->pvy_init ? pb->pvy_init[ii] : 0.0;
            } else if (c.igv.el[ii] >= Adhes) {
                c.igv.el[ii] = Adhes;                    // P=1: the normal part of the division
            }
        }
    }
    areas(c.igv);
    // coefficient of friction and shift of the previous time instance (P=0): copied for shifts,
    // carried one rolling step for rolling (gf3_dq_shift, m_gridfunc.f90:1864-1987) with the
    // static coefficient and zero shift beyond the grid; otherwise the static coefficient
    c.muv.assign(c.npot, c.fstat_eff);
    c.svx.assign(c.npot, 0.0); c.svy.assign(c.npot, 0.0);
    if (pb->pvtime == 0 && pb->mus_init) {
        const bool rolling = pb->tang == 2 || pb->tang == 3;
        int kx = 0; double facx = 0.0;
        if (rolling) {
            kx = (int)(c.dq * std::cos(c.chi) / dx);
            facx = c.dq * std::cos(c.chi) / dx - (double)(float)kx;
        }
        for (int iy = 0; iy < c.my; iy++)
            for (int ix = 0; ix < c.mx; ix++) {
                auto at = [&](const double *f, int jx, double ext) {
                    return (jx < 0 || jx >= c.mx) ? ext : f[jx + iy * c.mx];
                };
                const int ii = ix + iy * c.mx;
                c.muv[ii] = (1.0 - facx) * at(pb->mus_init, ix + kx, c.fstat_eff) + facx * at(pb->mus_init, ix + kx + 1, c.fstat_eff);
                if (pb->svx_init) {
                    c.svx[ii] = (1.0 - facx) * at(pb->svx_init, ix + kx, 0.0) + facx * at(pb->svx_init, ix + kx + 1, 0.0);
                    c.svy[ii] = (1.0 - facx) * at(pb->svy_init, ix + kx, 0.0) + facx * at(pb->svy_init, ix + kx + 1, 0.0);
                }
            }
    }
    init_curr_data(c, ihertz);
    // solver context
    TangCtx &tc = c.tc;
    tc.mx = c.mx; tc.my = c.my; tc.npot = c.npot; tc.dx = dx; tc.dy = dy; tc.dxdy = c.dxdy;
    tc.tang = pb->tang; tc.chi = c.chi; tc.dq = c.dq; tc.gausei_eff = pb->gausei;
    tc.maxgs = pb->maxgs; tc.maxin = pb->maxin; tc.eps = pb->eps;
    tc.omegah = pb->omegah; tc.omegas = pb->omegas;
    tc.kdowfb = pb->kdowfb; tc.fdecay = pb->fdecay; tc.betath = pb->betath;
    tc.d_ifc = pb->d_ifc; tc.d_lin = pb->d_lin; tc.d_cns = pb->d_cns; tc.d_slp = pb->d_slp; tc.pow_s = pb->pow_s;
    if (tc.d_lin * (tc.d_cns - tc.d_ifc) < 0.0) { tc.d_lin = 0.0; tc.d_cns = tc.d_ifc; }
    tc.kdown = 3;
    if (pb->gausei == 5) {
        if (tc.fdecay >= 0.999) tc.gd_meth = 1;
        else if (tc.fdecay <= 0.001) { tc.gd_meth = 2; tc.kdown = std::max(1, (int)std::nearbyint(-tc.fdecay)); }
        else tc.gd_meth = 3;
    } else {
        tc.gd_meth = 1;
    }
    // panprc, m_scontc.f90:356-553
    NormCtx nc{c.mx, c.my, c.npot, c.dxdy, pb->norm, c.fntrue};
    GF3 po1; po1.init(c.npot);
    gf_copy(AllElm, c.ps, po1, ikALL, c.igs);
    int itout = 0;
    double difid = 1.0, dif = 200.0 * difid;
    c.itnorm = 0; c.ittang = 0;
    while (dif > difid && itout < c.maxout && c.itnorm >= 0 && c.ittang >= 0) {
        itout++;
        int it;
        if (pb->bound >= 2 && pb->bound <= 4 && ihertz >= 1) {
            it = 0;
        } else {
            int itcg = 0;
            nc.fntrue = c.fntrue;
            it = snorm(nc, pb->maxgs, pb->maxin, pb->eps, c.cs, c.ms, c.hs, c.pen, c.igs, c.ps, itcg,
                       pb->sens, pb->mxsens, pb->epsens, &c.sens[iout_fn][iin_dpen]);
            c.itcg = itcg;
            if (it == -2) { c.aborted = true; break; }
            if (pb->norm == 0) c.fntrue = c.dxdy * gf_sum(AllElm, c.ps, ikZ, c.igs);
        }
        if (it >= 0) c.itnorm += it; else c.itnorm = -1;
        int ncon = 0;
        for (int ii = 0; ii < c.npot; ii++) {
            if (c.igs.el[ii] <= Exter) { c.ps.vn(ii) = 0; c.ps.vx(ii) = 0; c.ps.vy(ii) = 0; }
            else ncon++;
        }
        if (pb->tang == 0) {
            dif = 0.0;
        } else if (ncon <= 0) {
            dif = 0.0;
        } else {
            int itt = stang(c);
            if (c.unsupported || c.aborted) break;
            if (itt >= 0) c.ittang += itt; else c.ittang = -1;
            gf_axpy(AllElm, -1.0, c.ps, po1, ikALL, c.igs);
            dif = gf_rms(AllInt, po1, ikALL, c.igs);
            difid = 5.0 * pb->eps * gf_rms(AllInt, c.ps, ikALL, c.igs);
            if (r->nout < 64) { r->outer[2 * r->nout] = dif; r->outer[2 * r->nout + 1] = difid; }
            r->nout++;
            gf_copy(AllElm, c.ps, po1, ikALL, c.igs);
        }
    }
    r->mx = c.mx; r->my = c.my; r->dx = dx; r->dy = dy; r->xc1 = c.xc1; r->yc1 = c.yc1;
    r->a1 = c.a1; r->b1 = c.b1; r->aa = c.aa; r->bb = c.bb; r->rho = c.rho; r->cp = c.cp; r->aob = c.aob;
    r->cksi = c.cksi; r->ceta = c.ceta; r->cphi = c.cphi;
    r->itnorm = c.itnorm; r->ittang = c.ittang; r->itcg = c.itcg; r->itgs = c.itgs; r->solver = c.solver_eff;
    for (int io = 0; io < 4; io++)
        for (int ji = 0; ji < 4; ji++) r->sens[io + 4 * ji] = c.sens[io][ji];
    r->nslp = (int)(c.slp_hist.size() / 4);
    for (int q = 0; q < std::min(r->nslp, 64) * 4; q++) r->slp[q] = c.slp_hist[q];
    r->nnr = (int)(c.nr_hist.size() / 7);
    if (r->nr_hist)
        for (int q = 0; q < std::min(r->nnr, r->nr_cap) * 7; q++) r->nr_hist[q] = c.nr_hist[q];
    if (c.unsupported || c.aborted) { r->ierror = CNTC_err_other; return r->ierror; }
    soutpt(c, r);
    r->pen = c.pen;
    for (int ii = 0; ii < c.npot; ii++) {
        if (r->pn) r->pn[ii] = c.ps.vn(ii);
        if (r->px) r->px[ii] = c.ps.vx(ii);
        if (r->py) r->py[ii] = c.ps.vy(ii);
        if (r->un) r->un[ii] = c.us.vn(ii);
        if (r->ux) r->ux[ii] = c.us.vx(ii);
        if (r->uy) r->uy[ii] = c.us.vy(ii);
        if (r->sx) r->sx[ii] = c.ss.vx(ii) / c.dq;
        if (r->sy) r->sy[ii] = c.ss.vy(ii) / c.dq;
        if (r->h) r->h[ii] = c.hs.vn(ii);
        if (r->igs) r->igs[ii] = c.igs.el[ii];
        if (r->mus) r->mus[ii] = c.mus[ii];
    }
    if (c.itnorm < 0) r->ierror = CNTC_err_norm;
    else if (c.ittang < 0) r->ierror = CNTC_err_tang;
    else r->ierror = eldiv_count_atbnd(c.igs);
    return r->ierror;
}

} // extern "C"
