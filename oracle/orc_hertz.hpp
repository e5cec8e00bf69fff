// CPU ORACLE -- test infrastructure only (see contact_oracle.h).
//
// 3-D Hertz solution (src/m_hertz.f90).  The complete elliptic integrals K(k), E(k)
// and the associate integrals B = K - D, D = (K - E)/k^2 are evaluated with
// Carlson's symmetric forms R_F and R_D by the duplication theorem
// (B.C. Carlson, "Numerical computation of real or complex elliptic integrals",
// Numer. Algorithms 10 (1995)); the reference uses Fukushima's (2011) series for
// the same quantities.
#pragma once
#include "orc_core.hpp"

namespace orc {

inline double carlson_rf(double x, double y, double z) {
    for (int it = 0; it < 200; it++) {
        double mu = (x + y + z) / 3.0;
        double dx = 1.0 - x / mu, dy = 1.0 - y / mu, dz = 1.0 - z / mu;
        if (std::max(std::fabs(dx), std::max(std::fabs(dy), std::fabs(dz))) < 1e-4) {
            double e2 = dx * dy - dz * dz, e3 = dx * dy * dz;
            return (1.0 - e2 / 10.0 + e3 / 14.0 + e2 * e2 / 24.0 - 3.0 * e2 * e3 / 44.0) / std::sqrt(mu);
        }
        double sx = std::sqrt(x), sy = std::sqrt(y), sz = std::sqrt(z);
        double lam = sx * sy + sy * sz + sz * sx;
        x = 0.25 * (x + lam); y = 0.25 * (y + lam); z = 0.25 * (z + lam);
    }
    return 1.0 / std::sqrt((x + y + z) / 3.0);
}

inline double carlson_rd(double x, double y, double z) {
    double sum = 0.0, fac = 1.0;
    for (int it = 0; it < 200; it++) {
        double mu = (x + y + 3.0 * z) / 5.0;
        double dx = (mu - x) / mu, dy = (mu - y) / mu, dz = (mu - z) / mu;
        if (std::max(std::fabs(dx), std::max(std::fabs(dy), std::fabs(dz))) < 1e-4) {
            double ea = dx * dy, eb = dz * dz, ec = ea - eb, ed = ea - 6.0 * eb, ee = ed + ec + ec;
            double s = 1.0 + ed * (-3.0 / 14.0 + 9.0 / 88.0 * ed - 9.0 / 52.0 * dz * ee)
                     + dz * (ee / 6.0 + dz * (-9.0 / 22.0 * ec + 3.0 / 26.0 * dz * ea));
            return 3.0 * sum + fac * s / (mu * std::sqrt(mu));
        }
        double sx = std::sqrt(x), sy = std::sqrt(y), sz = std::sqrt(z);
        double lam = sx * sy + sy * sz + sz * sx;
        sum += fac / (sz * (z + lam));
        fac *= 0.25;
        x = 0.25 * (x + lam); y = 0.25 * (y + lam); z = 0.25 * (z + lam);
    }
    double mu = (x + y + 3.0 * z) / 5.0;
    return 3.0 * sum + fac / (mu * std::sqrt(mu));
}

// eli, m_hertz.f90:447-499: returns the curvature ratio (E - B)/B for modulus k and K, E
inline double eli(double elmodk, double &ell_k, double &ell_e) {
    double mc = 1.0 - elmodk * elmodk;
    if (mc <= 1e-300) { ell_k = 1e300; ell_e = 1.0; return 0.0; }
    double rf = carlson_rf(0.0, mc, 1.0);
    double d = carlson_rd(0.0, mc, 1.0) / 3.0;
    double b = rf - d;
    ell_k = b + d;
    ell_e = b + mc * d;
    return (ell_e - b) / b;
}

// bisec, m_hertz.f90:390-443
inline void bisec(double &ellk, double &elle, double epshz, double &x, double xlft, double xrght, double y) {
    double xl = xlft, xr = xrght;
    double elr = eli(xr, ellk, elle);
    double ell = eli(xl, ellk, elle);
    (void)ell;
    x = 0.5 * (xl + xr);
    while (std::fabs(xr - xl) > epshz) {
        x = (xl + xr) / 2.0;
        double elx = eli(x, ellk, elle);
        if ((y - elr) * (y - elx) <= 0.0) { xl = x; ell = elx; }
        else { xr = x; elr = elx; }
    }
    eli(x, ellk, elle);
}

// hzcalc3d, m_hertz.f90:267-384
inline void hzcalc3d(double e_star, double epshz, int ipotcn, double &a1, double &b1, double &aa, double &bb,
                     int ic_norm, double &pen, double &fntrue, double &cp, double &rho) {
    const double penmin = 1e-9;
    double ellipk, ellipe, g, sqrtg, elmodk, y, x;
    bool zbla;
    if (ipotcn == -1) {
        zbla = (b1 <= a1);
        y = zbla ? b1 / a1 : a1 / b1;
        bisec(ellipk, ellipe, epshz, x, 0.0, 1.0, y);
        elmodk = x;
        g = std::sqrt(std::max(1e-40, 1.0 - elmodk * elmodk));
        sqrtg = std::sqrt(g);
        rho = 2.0 / (a1 + b1);
        if (ic_norm == 1) {
            cp = std::pow((3.0 * std::max(0.0, fntrue) * rho * ellipe) / (4.0 * pi * e_star * sqrtg), 1.0 / 3.0);
            pen = 2.0 * (cp * sqrtg) * (cp * sqrtg) * ellipk / (rho * ellipe);
        } else {
            cp = std::sqrt((std::max(0.0, pen) * rho * ellipe) / (2.0 * ellipk * sqrtg * sqrtg));
            fntrue = 4.0 * pi * cp * cp * cp * e_star * sqrtg / (3.0 * rho * ellipe);
        }
        if (zbla) { aa = cp * sqrtg; bb = cp / sqrtg; }
        else      { aa = cp / sqrtg; bb = cp * sqrtg; }
    } else {
        zbla = (bb <= aa);
        g = zbla ? bb / aa : aa / bb;
        sqrtg = std::sqrt(g);
        elmodk = std::sqrt(1.0 - g * g);
        y = eli(elmodk, ellipk, ellipe);
        cp = std::sqrt(aa * bb);
        if (ic_norm == 1) {
            rho = 4.0 * pi * cp * cp * cp * e_star * sqrtg / (3.0 * fntrue * ellipe);
            pen = 2.0 * (cp * sqrtg) * (cp * sqrtg) * ellipk / (rho * ellipe);
        } else {
            pen = std::max(pen, penmin);
            rho = 2.0 * (cp * sqrtg) * (cp * sqrtg) * ellipk / (pen * ellipe);
            fntrue = 4.0 * pi * cp * cp * cp * e_star * sqrtg / (3.0 * rho * ellipe);
        }
        double apb = 2.0 / rho, ama = apb / (y + 1.0), ami = y * ama;
        if (zbla) { a1 = ami; b1 = ama; } else { a1 = ama; b1 = ami; }
    }
}

// elliptic_to_curv, m_hertz.f90:97-207 (regula falsi on b1 for a prescribed a/b)
inline void elliptic_to_curv(int ic_norm, double &a1, double &aa, double aob, double &b1, double &bb, double &cp,
                             double &rho, double &fntrue, double &pen, double e_star, double epshz) {
    double epsaob = 10.0 * epshz;
    int ipotcn = -1, iter = 0;
    b1 = a1;
    hzcalc3d(e_star, epshz, ipotcn, a1, b1, aa, bb, ic_norm, pen, fntrue, cp, rho);
    if (aa < tiny_ && bb < tiny_) return;
    double b1low, b1high, aoblow, aobhigh;
    if (aa / bb > aob) {
        b1high = b1; aobhigh = aa / bb;
        while (iter <= 100 && aa / bb > aob) {
            iter++; b1high = b1; aobhigh = aa / bb; b1 = b1 * 0.5;
            hzcalc3d(e_star, epshz, ipotcn, a1, b1, aa, bb, ic_norm, pen, fntrue, cp, rho);
        }
        b1low = b1; aoblow = aa / bb;
    } else {
        b1low = b1; aoblow = aa / bb;
        while (iter <= 100 && aa / bb < aob) {
            iter++; b1low = b1; aoblow = aa / bb; b1 = b1 * 2.0;
            hzcalc3d(e_star, epshz, ipotcn, a1, b1, aa, bb, ic_norm, pen, fntrue, cp, rho);
        }
        b1high = b1; aobhigh = aa / bb;
    }
    while (iter <= 100 && std::fabs(aa / bb - aob) > epsaob * aob) {
        iter++;
        double daob = aob - aoblow;
        double rico = (aobhigh - aoblow) / (b1high - b1low);
        b1 = b1low + daob / rico;
        hzcalc3d(e_star, epshz, ipotcn, a1, b1, aa, bb, ic_norm, pen, fntrue, cp, rho);
        if (aa / bb > aob) { b1high = b1; aobhigh = aa / bb; }
        else { b1low = b1; aoblow = aa / bb; }
    }
}

} // namespace orc
