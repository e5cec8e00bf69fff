// CPU ORACLE -- test infrastructure only (see contact_oracle.h).
//
// Single-element tangential solver plstrc / elmtrc (m_solvpt.f90:3258-3807), used by
// SteadyGS and by GDsteady's diagonal scaling and local optimisation.
#pragma once
#include "orc_core.hpp"

namespace orc {

// plstrc, m_solvpt.f90:3278-3807.  coef is column-major coef(i,j) -> coef[i-1][j-1].
inline void plstrc(int &el, const double coef[2][2], double eps, double omegah, double omegas,
                   double pr[3], double mus, bool use_plast, double tau_c0, double k_tau,
                   double taucv, double &taucs, double s[2], double dupl[2]) {
    const int maxnr = 10;
    const double prc = 0.0001;
    if (!use_plast) taucs = 1e20;
    double pold1 = pr[0], pold2 = pr[1];
    double si0[2], si[2] = {0, 0}, dp[2], fk[2], gradf[2][2];
    si0[0] = s[0] - coef[0][0] * pr[0] - coef[0][1] * pr[1];
    si0[1] = s[1] - coef[1][0] * pr[0] - coef[1][1] * pr[1];
    int itry = 0, violat = 1;
    double trc_bound = 0.0, dupl_abs = 0.0;
    while (itry <= 3 && violat == 1) {
        itry++;
        if (el == Adhes) {
            dupl[0] = 0.0; dupl[1] = 0.0;
            if (use_plast) taucs = taucv;
            trc_bound = mus * pr[2];
            double detinv = 1.0 / (coef[0][0] * coef[1][1] - coef[0][1] * coef[1][0]);
            dp[0] = (-coef[1][1] * s[0] + coef[0][1] * s[1]) * detinv;
            dp[1] = (coef[1][0] * s[0] - coef[0][0] * s[1]) * detinv;
            pr[0] = pold1 + omegah * dp[0];
            pr[1] = pold2 + omegah * dp[1];
            double pabs2 = std::sqrt(pr[0] * pr[0] + pr[1] * pr[1]);
            double bnd = std::min(trc_bound, taucs);
            if (pabs2 <= bnd) {
                violat = 0;
            } else {
                double pabs1 = std::sqrt((pold1 + dp[0]) * (pold1 + dp[0]) + (pold2 + dp[1]) * (pold2 + dp[1]));
                if (pabs1 <= bnd) {
                    pr[0] = pr[0] * bnd / pabs2; pr[1] = pr[1] * bnd / pabs2;
                    violat = 0;
                } else {
                    violat = 1;
                }
            }
            si[0] = si0[0] + coef[0][0] * pr[0] + coef[0][1] * pr[1];
            si[1] = si0[1] + coef[1][0] * pr[0] + coef[1][1] * pr[1];
        } else if (el == Slip) {
            violat = 0;
            trc_bound = mus * pr[2];
            dupl[0] = 0.0; dupl[1] = 0.0;
            if (use_plast) taucs = taucv;
            double sabs = std::sqrt(si0[0] * si0[0] + si0[1] * si0[1]);
            pr[0] = -trc_bound * si0[0] / sabs;
            pr[1] = -trc_bound * si0[1] / sabs;
            si[0] = si0[0] + coef[0][0] * pr[0] + coef[0][1] * pr[1];
            si[1] = si0[1] + coef[1][0] * pr[0] + coef[1][1] * pr[1];
            fk[0] = pr[1] * si[0] - pr[0] * si[1];
            fk[1] = pr[0] * pr[0] + pr[1] * pr[1] - trc_bound * trc_bound;
            int itnr = 0;
            while (itnr == 0 || (itnr < maxnr && std::fabs(fk[0]) + std::fabs(fk[1]) >= prc * eps * trc_bound)) {
                itnr++;
                gradf[0][0] = -2.0 * coef[1][0] * pr[0] - si0[1] + (coef[0][0] - coef[1][1]) * pr[1];
                gradf[0][1] = 2.0 * coef[0][1] * pr[1] + si0[0] + (coef[0][0] - coef[1][1]) * pr[0];
                gradf[1][0] = 2.0 * pr[0];
                gradf[1][1] = 2.0 * pr[1];
                double det = gradf[0][0] * gradf[1][1] - gradf[0][1] * gradf[1][0];
                if (det == 0.0) {
                    itnr = maxnr;
                } else {
                    dp[0] = -(gradf[1][1] * fk[0] - gradf[0][1] * fk[1]) / det;
                    dp[1] = -(-gradf[1][0] * fk[0] + gradf[0][0] * fk[1]) / det;
                    pr[0] += dp[0]; pr[1] += dp[1];
                }
                si[0] = si0[0] + coef[0][0] * pr[0] + coef[0][1] * pr[1];
                si[1] = si0[1] + coef[1][0] * pr[0] + coef[1][1] * pr[1];
                fk[0] = pr[1] * si[0] - pr[0] * si[1];
                fk[1] = pr[0] * pr[0] + pr[1] * pr[1] - trc_bound * trc_bound;
            }
            double alph0 = std::atan2(pold2, pold1);
            double alph1 = std::atan2(pr[1], pr[0]);
            double dalph = alph1 - alph0;
            if (dalph < -pi) dalph += 2.0 * pi;
            if (dalph > pi) dalph -= 2.0 * pi;
            alph1 = alph0 + omegas * dalph;
            pr[0] = trc_bound * std::cos(alph1);
            pr[1] = trc_bound * std::sin(alph1);
            if (taucs < trc_bound) {
                if (k_tau < 0.0) violat = 1;
                taucs = trc_bound;
                double pabs2 = std::sqrt(pr[0] * pr[0] + pr[1] * pr[1]);
                dupl[0] = (taucs - taucv) * pr[0] / (pabs2 * k_tau);
                dupl[1] = (taucs - taucv) * pr[1] / (pabs2 * k_tau);
                si[0] += dupl[0]; si[1] += dupl[1];
            }
            if (std::fabs(pr[0]) > std::fabs(pr[1])) { if (pr[0] * si[0] > 0.0) violat = 1; }
            else { if (pr[1] * si[1] > 0.0) violat = 1; }
        } else {
            trc_bound = mus * pr[2];
            si[0] = 0.0; si[1] = 0.0;
            if (use_plast) taucs = taucv;
            double theta = std::atan2(-si0[1], -si0[0]);
            double theta_prv = 0.0;
            int itnr = 0;
            while (itnr == 0 || (itnr < maxnr && std::fabs(theta - theta_prv) >= eps)) {
                itnr++;
                theta_prv = theta;
                double cs = std::cos(theta), sn = std::sin(theta);
                pr[0] = taucs * cs; pr[1] = taucs * sn;
                double ws0 = si0[0] + coef[0][0] * pr[0] + coef[0][1] * pr[1];
                double ws1 = si0[1] + coef[1][0] * pr[0] + coef[1][1] * pr[1];
                dupl_abs = -(ws0 * cs + ws1 * sn) /
                           (((coef[0][0] * cs + coef[0][1] * sn) * cs + (coef[1][0] * cs + coef[1][1] * sn) * sn) * k_tau + 1.0);
                if (dupl_abs < 0.0) dupl_abs = 0.0;
                dupl[0] = dupl_abs * cs; dupl[1] = dupl_abs * sn;
                pr[0] += dupl[0] * k_tau; pr[1] += dupl[1] * k_tau;
                double uel0 = coef[0][0] * pr[0] + coef[0][1] * pr[1];
                double uel1 = coef[1][0] * pr[0] + coef[1][1] * pr[1];
                double ut0 = uel0 + dupl[0], ut1 = uel1 + dupl[1];
                double theta_given = theta;
                double theta_eff = std::atan2(ut1, ut0);
                double theta_tgt = std::atan2(-si0[1], -si0[0]);
                double det = coef[0][0] * coef[1][1] - coef[0][1] * coef[1][0];
                double dfdx = det / ((coef[1][1] * coef[1][1] + coef[0][1] * coef[0][1]) * sn * sn +
                                     2 * (coef[1][0] * coef[1][1] + coef[0][0] * coef[0][1]) * cs * sn +
                                     (coef[1][0] * coef[1][0] + coef[0][0] * coef[0][0]) * cs * cs);
                theta = theta_given - (theta_eff - theta_tgt) / dfdx;
            }
            if (use_plast) taucs = taucv + k_tau * dupl_abs;
            taucs = std::max(0.1 * tau_c0, taucs);
            violat = 0;
            if (dupl_abs <= tiny_) violat = 1;
            if (std::fabs(pr[0]) > std::fabs(pr[1])) { if (pr[0] * dupl[0] < 0.0) violat = 1; }
            else { if (pr[1] * dupl[1] < 0.0) violat = 1; }
            if (taucs >= trc_bound) violat = 1;
        }
        if (itry <= 3 && violat == 1) {
            if (el == Adhes) el = (k_tau > 0.0 || trc_bound <= taucs) ? Slip : Plast;
            else if (el == Slip) el = Plast;
            else el = Adhes;
        }
    }
    s[0] = si[0]; s[1] = si[1];
}

// elmtrc, m_solvpt.f90:3258-3274
inline void elmtrc(int &el, const double coef[2][2], double eps, double omegah, double omegas,
                   double pr[3], double mus, double s[2]) {
    const double tau_c0 = 1e20, taucv = 1e20, k_tau = 0.0;
    double taucs = taucv, dupl[2];
    plstrc(el, coef, eps, omegah, omegas, pr, mus, false, tau_c0, k_tau, taucv, taucs, s, dupl);
}

} // namespace orc
