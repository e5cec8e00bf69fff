// Host-side Hertz solution for the library (src/m_hertz.f90:29-384): semi-axes, curvatures,
// approach and effective radius for elliptic Hertzian contact.  The complete elliptic
// integrals are obtained from Carlson's symmetric integrals R_F and R_D by the duplication
// theorem (B.C. Carlson, Numer. Algorithms 10, 1995).
#pragma once
#include <algorithm>
#include <cmath>

namespace cgb {
namespace hz {

inline double rf(double x, double y, double z) {
    for (int it = 0; it < 200; it++) {
        const double mu = (x + y + z) / 3.0;
        const double ex = 1.0 - x / mu, ey = 1.0 - y / mu, ez = 1.0 - z / mu;
        if (std::max(std::fabs(ex), std::max(std::fabs(ey), std::fabs(ez))) < 1e-4) {
            const double e2 = ex * ey - ez * ez, e3 = ex * ey * ez;
            return (1.0 - e2 / 10.0 + e3 / 14.0 + e2 * e2 / 24.0 - 3.0 * e2 * e3 / 44.0) / std::sqrt(mu);
        }
        const double l = std::sqrt(x) * std::sqrt(y) + std::sqrt(y) * std::sqrt(z) + std::sqrt(z) * std::sqrt(x);
        x = 0.25 * (x + l); y = 0.25 * (y + l); z = 0.25 * (z + l);
    }
    return 1.0 / std::sqrt((x + y + z) / 3.0);
}

inline double rd(double x, double y, double z) {
    double acc = 0.0, f = 1.0;
    for (int it = 0; it < 200; it++) {
        const double mu = (x + y + 3.0 * z) / 5.0;
        const double ex = (mu - x) / mu, ey = (mu - y) / mu, ez = (mu - z) / mu;
        if (std::max(std::fabs(ex), std::max(std::fabs(ey), std::fabs(ez))) < 1e-4) {
            const double ea = ex * ey, eb = ez * ez, ec = ea - eb, ed = ea - 6.0 * eb, ee = ed + ec + ec;
            const double s = 1.0 + ed * (-3.0 / 14.0 + 9.0 / 88.0 * ed - 9.0 / 52.0 * ez * ee) +
                             ez * (ee / 6.0 + ez * (-9.0 / 22.0 * ec + 3.0 / 26.0 * ez * ea));
            return 3.0 * acc + f * s / (mu * std::sqrt(mu));
        }
        const double sz = std::sqrt(z);
        const double l = std::sqrt(x) * std::sqrt(y) + std::sqrt(y) * sz + sz * std::sqrt(x);
        acc += f / (sz * (z + l));
        f *= 0.25;
        x = 0.25 * (x + l); y = 0.25 * (y + l); z = 0.25 * (z + l);
    }
    const double mu = (x + y + 3.0 * z) / 5.0;
    return 3.0 * acc + f / (mu * std::sqrt(mu));
}

// curvature ratio (E - B)/B for elliptic modulus k, with K(k), E(k)
inline double curv_ratio(double k, double &K, double &E) {
    const double mc = 1.0 - k * k;
    if (mc <= 1e-300) { K = 1e300; E = 1.0; return 0.0; }
    const double f = rf(0.0, mc, 1.0);
    const double d = rd(0.0, mc, 1.0) / 3.0;
    const double b = f - d;
    K = f;
    E = b + mc * d;
    return (E - b) / b;
}

struct Result {
    double a1, b1, aa, bb, cp, rho, pen, fn;
};

// 3-D Hertz with semi-axes (ipotcn -3) or curvatures (ipotcn -1) prescribed, normal force
// (norm = 1) or approach (norm = 0) prescribed; e_star = G / (1 - nu)
inline void calc3d(double e_star, int ipotcn, int norm, Result &r) {
    const double pi = 3.14159265358979323846, epshz = (double)1e-9f;
    double K, E, g, sqg;
    if (ipotcn == -1) {
        const bool b_le_a = r.b1 <= r.a1;
        const double y = b_le_a ? r.b1 / r.a1 : r.a1 / r.b1;
        double lo = 0.0, hi = 1.0, x = 0.5;
        double fhi = curv_ratio(hi, K, E);
        curv_ratio(lo, K, E);
        while (std::fabs(hi - lo) > epshz) {
            x = 0.5 * (lo + hi);
            const double fx = curv_ratio(x, K, E);
            if ((y - fhi) * (y - fx) <= 0.0) lo = x;
            else { hi = x; fhi = fx; }
        }
        curv_ratio(x, K, E);
        g = std::sqrt(std::max(1e-40, 1.0 - x * x));
        sqg = std::sqrt(g);
        r.rho = 2.0 / (r.a1 + r.b1);
        if (norm == 1) {
            r.cp = std::pow((3.0 * std::max(0.0, r.fn) * r.rho * E) / (4.0 * pi * e_star * sqg), 1.0 / 3.0);
            r.pen = 2.0 * (r.cp * sqg) * (r.cp * sqg) * K / (r.rho * E);
        } else {
            r.cp = std::sqrt((std::max(0.0, r.pen) * r.rho * E) / (2.0 * K * sqg * sqg));
            r.fn = 4.0 * pi * r.cp * r.cp * r.cp * e_star * sqg / (3.0 * r.rho * E);
        }
        if (b_le_a) { r.aa = r.cp * sqg; r.bb = r.cp / sqg; }
        else { r.aa = r.cp / sqg; r.bb = r.cp * sqg; }
    } else {
        const bool b_le_a = r.bb <= r.aa;
        g = b_le_a ? r.bb / r.aa : r.aa / r.bb;
        sqg = std::sqrt(g);
        const double y = curv_ratio(std::sqrt(1.0 - g * g), K, E);
        r.cp = std::sqrt(r.aa * r.bb);
        if (norm == 1) {
            r.rho = 4.0 * pi * r.cp * r.cp * r.cp * e_star * sqg / (3.0 * r.fn * E);
            r.pen = 2.0 * (r.cp * sqg) * (r.cp * sqg) * K / (r.rho * E);
        } else {
            r.pen = std::max(r.pen, 1e-9);
            r.rho = 2.0 * (r.cp * sqg) * (r.cp * sqg) * K / (r.pen * E);
            r.fn = 4.0 * pi * r.cp * r.cp * r.cp * e_star * sqg / (3.0 * r.rho * E);
        }
        const double amax = (2.0 / r.rho) / (y + 1.0), amin = y * amax;
        if (b_le_a) { r.a1 = amin; r.b1 = amax; } else { r.a1 = amax; r.b1 = amin; }
    }
}

// curvature a1 and ellipticity aa/bb prescribed (ipotcn -2): regula falsi on b1
inline void calc_aob(double e_star, int norm, double aob, Result &r) {
    const double epsaob = 10.0 * (double)1e-9f;
    int iter = 0;
    r.b1 = r.a1;
    calc3d(e_star, -1, norm, r);
    if (r.aa < 1e-20 && r.bb < 1e-20) return;
    double blo, bhi, qlo, qhi;
    if (r.aa / r.bb > aob) {
        bhi = r.b1; qhi = r.aa / r.bb;
        while (iter <= 100 && r.aa / r.bb > aob) {
            iter++; bhi = r.b1; qhi = r.aa / r.bb; r.b1 *= 0.5;
            calc3d(e_star, -1, norm, r);
        }
        blo = r.b1; qlo = r.aa / r.bb;
    } else {
        blo = r.b1; qlo = r.aa / r.bb;
        while (iter <= 100 && r.aa / r.bb < aob) {
            iter++; blo = r.b1; qlo = r.aa / r.bb; r.b1 *= 2.0;
            calc3d(e_star, -1, norm, r);
        }
        bhi = r.b1; qhi = r.aa / r.bb;
    }
    while (iter <= 100 && std::fabs(r.aa / r.bb - aob) > epsaob * aob) {
        iter++;
        r.b1 = blo + (aob - qlo) / ((qhi - qlo) / (bhi - blo));
        calc3d(e_star, -1, norm, r);
        if (r.aa / r.bb > aob) { bhi = r.b1; qhi = r.aa / r.bb; }
        else { blo = r.b1; qlo = r.aa / r.bb; }
    }
}

} // namespace hz
} // namespace cgb
