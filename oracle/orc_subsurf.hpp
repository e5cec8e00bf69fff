// CPU ORACLE -- test infrastructure only (see contact_oracle.h).
//
// Subsurface elastic field of the surface tractions (m_subsurf.f90): the displacements and
// displacement gradients below a uniformly loaded rectangle (stres1_pcwcns, :1633-1852, after
// Kalker, "Numerical calculation of the elastic field in a half-space", Comm. Appl. Num. Meth.
// 2, 1986, 401-410), their sum over the loaded elements at arbitrary points (sstres,
// :1412-1515), the same at element centres by per-depth influence coefficients and FFT
// convolution (sstres_inflcf :1261-1408, sstres_fft :1097-1257), and the stresses, invariants
// and principal stresses derived from them (sstres_derived, :1519-1629).  Piecewise-constant
// tractions only (C=2).
#pragma once
#include "orc_conv.hpp"

namespace orc {

// Displacements v[i][j][0] in direction j and their gradients v[i][j][k] (d/dx_k) at xw due to
// a unit traction in direction i on the dx x dy element centred at xp; vnu holds the parts
// proportional to Poisson's ratio.  Requires xw[2] >= 0.
inline void stres1_pcwcns(double dx, double dy, double gg, double v[3][3][4], double vnu[3][3][4],
                          const double xw[3], const double xp[2]) {
    const double epsrel = 5e-7;
    static const int sgn[3] = {-1, -1, 1};
    static const int ip[3] = {1, 2, 0};                  // next direction (0-based)
    auto kd = [](int a, int b) { return a == b ? 1.0 : 0.0; };
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            for (int k = 0; k < 4; k++) { v[i][j][k] = 0.0; vnu[i][j][k] = 0.0; }
    for (int jx = -1; jx <= 1; jx += 2)
        for (int jy = -1; jy <= 1; jy += 2) {
            double y[3] = {xp[0] + jx * dx / 2.0 - xw[0], xp[1] + jy * dy / 2.0 - xw[1], xw[2]};
            const double w = std::max(1e-12, std::sqrt(y[0] * y[0] + y[1] * y[1] + y[2] * y[2]));
            // perturbed components, |yeps_i| >= epsrel w with the sign of y_i, so that weps - yeps_i > 0
            const double epsy = epsrel * w;
            double ye[3];
            for (int i = 0; i < 3; i++) ye[i] = (y[i] >= 0.0) ? std::max(epsy, y[i]) : std::min(-epsy, y[i]);
            const double we = std::max(1e-12, std::sqrt(ye[0] * ye[0] + ye[1] * ye[1] + ye[2] * ye[2]));
            double al[3], at[3], wm[4];
            wm[0] = we;
            for (int k = 0; k < 3; k++) {
                al[k] = std::log(y[k] + we);
                at[k] = std::atan((y[ip[k]] + y[ip[ip[k]]] + w) / ye[k]);
                wm[k + 1] = sgn[k] * y[k] / we;
            }
            double a[3][3][4], t[3][3][4];
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++) {
                    a[i][j][0] = y[i] * al[j];
                    t[i][j][0] = y[i] * at[j];
                    for (int k = 0; k < 3; k++) {
                        a[i][j][k + 1] = sgn[k] * (kd(i, k) * al[j] + y[i] * (kd(j, k) * w + y[k]) / (we * (y[j] + we)));
                        t[i][j][k + 1] = sgn[k] * (kd(i, k) * at[j] +
                                                   y[i] * (y[j] * (y[k] + w) - kd(j, k) * w * (y[0] + y[1] + y[2] + w)) /
                                                       (2 * we * (y[ip[j]] + we) * (y[ip[ip[j]]] + we)));
                    }
                }
            const double s = jx * jy;
            for (int k = 0; k < 4; k++) {
                for (int i = 0; i < 2; i++) {
                    const int l = 1 - i;
                    double q = a[i][l][k] + 2 * a[l][i][k] + 4 * t[2][2][k] + a[i][l][k] - 2 * t[2][i][k];
                    v[i][i][k] += s * q;
                    q = -2 * (a[i][l][k] - 2 * t[2][i][k]);
                    vnu[i][i][k] += q * s;
                    q = -a[2][2][k];
                    v[i][l][k] += s * q;
                    q = 2 * (a[2][2][k] - wm[k]);
                    vnu[i][l][k] += q * s;
                    q = 2 * (a[l][2][k] + a[2][l][k] + 2 * t[i][i][k]);
                    vnu[i][2][k] += q * s;
                    vnu[2][i][k] = -vnu[i][2][k];
                    q = -a[l][2][k] - 2 * t[i][i][k];
                    v[i][2][k] += q * s;
                    v[2][i][k] += (2 * a[2][l][k] - q) * s;
                }
                double q = -2 * (a[0][1][k] + a[1][0][k] + 2 * t[2][2][k]);
                vnu[2][2][k] += q * s;
                q = -2 * t[2][2][k] + 2 * (a[0][1][k] + a[1][0][k] + 2 * t[2][2][k]);
                v[2][2][k] += q * s;
            }
        }
    const double f = 4.0 * pi * gg;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            for (int k = 0; k < 4; k++) { v[i][j][k] /= f; vnu[i][j][k] /= f; }
}

// Eigenvalues of a symmetric 3x3 matrix, largest first, by the trigonometric solution of its
// characteristic cubic (O. K. Smith, "Eigenvalues of a symmetric 3x3 matrix", Comm. ACM 4,
// 1961, 168).  The reference uses an analytic 3x3 solver too (dsyevc3); both agree to rounding.
inline void sym3_eigenvalues(const double s[3][3], double ev[3]) {
    const double p1 = s[0][1] * s[0][1] + s[0][2] * s[0][2] + s[1][2] * s[1][2];
    const double q = (s[0][0] + s[1][1] + s[2][2]) / 3.0;
    const double d0 = s[0][0] - q, d1 = s[1][1] - q, d2 = s[2][2] - q;
    const double p2 = d0 * d0 + d1 * d1 + d2 * d2 + 2.0 * p1;
    if (p2 <= 0.0) { ev[0] = ev[1] = ev[2] = q; return; }
    const double p = std::sqrt(p2 / 6.0);
    const double b00 = d0 / p, b11 = d1 / p, b22 = d2 / p, b01 = s[0][1] / p, b02 = s[0][2] / p, b12 = s[1][2] / p;
    double r = 0.5 * (b00 * (b11 * b22 - b12 * b12) - b01 * (b01 * b22 - b12 * b02) + b02 * (b01 * b12 - b11 * b02));
    r = std::max(-1.0, std::min(1.0, r));
    const double phi = std::acos(r) / 3.0;
    ev[0] = q + 2.0 * p * std::cos(phi);
    ev[2] = q + 2.0 * p * std::cos(phi + 2.0 * pi / 3.0);
    ev[1] = 3.0 * q - ev[0] - ev[2];
}

// One subsurface result: displacements, stress tensor, principal stresses (largest first),
// hydrostatic, von Mises and Tresca stresses
struct SubsPoint {
    double u[3], sig[3][3], sigmaj[3], sighyd, sigvm, sigtr;
};

// sstres_derived, m_subsurf.f90:1519-1629: the mirrored components for body 2 (neg = -1),
// linearised strain, Hooke's law, invariants; values below gg 1e-15 set to zero
inline SubsPoint sstres_derived(double gg, double poiss, int neg, double vr[3][4]) {
    const double tolsml = 1e-15;
    SubsPoint r;
    for (int j = 0; j < 3; j++) {
        const int fj = (j == 1 || j == 2) ? neg : 1;
        for (int k = 0; k < 4; k++) {
            const int fk = (k == 2 || k == 3) ? neg : 1;
            vr[j][k] = fj * fk * vr[j][k];
        }
    }
    for (int i = 0; i < 3; i++) r.u[i] = vr[i][0];
    double er[3][3];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) er[i][j] = (vr[i][j + 1] + vr[j][i + 1]) / 2.0;
    const double dil = er[0][0] + er[1][1] + er[2][2];
    for (int j = 0; j < 3; j++)
        for (int i = 0; i < 3; i++) r.sig[i][j] = 2.0 * gg * er[i][j];
    for (int i = 0; i < 3; i++) r.sig[i][i] += 2.0 * gg * dil * poiss / std::max(1e-6, 1.0 - 2.0 * poiss);
    const double sigii = r.sig[0][0] + r.sig[1][1] + r.sig[2][2];
    r.sighyd = sigii / 3.0;
    double sijsij = -(1.0 / 3.0) * sigii * sigii;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) sijsij += r.sig[i][j] * r.sig[i][j];
    sijsij = 0.5 * sijsij;
    r.sigvm = std::sqrt(3.0 * sijsij);
    sym3_eigenvalues(r.sig, r.sigmaj);
    r.sigtr = r.sigmaj[0] - r.sigmaj[2];
    for (int i = 0; i < 3; i++)
        if (std::fabs(r.u[i]) < gg * tolsml) r.u[i] = 0.0;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            if (std::fabs(r.sig[i][j]) < gg * tolsml) r.sig[i][j] = 0.0;
    return r;
}

// Tractions on the surface grid: element centres (x fastest), spacing and the tractions of
// body 1 (pn, px, py); gg[0..1], poiss[0..1] the two bodies (z >= 0 body 1, z < 0 body 2)
struct SubsLoad {
    int mx, my;
    double dx, dy, xc1, yc1;
    const double *pn, *px, *py;
    double gg[2], poiss[2];
};

// sstres, m_subsurf.f90:1412-1515: the field at one point, summed over the elements with
// positive pressure
inline SubsPoint sstres_point(const SubsLoad &L, const double xw_in[3]) {
    double xw[3] = {xw_in[0], xw_in[1], xw_in[2]};
    const int ia = (xw[2] >= 0.0) ? 0 : 1, neg = (xw[2] >= 0.0) ? 1 : -1;
    xw[2] = neg * xw[2];
    xw[1] = neg * xw[1];
    double vr[3][4] = {};
    double v[3][3][4], vnu[3][3][4];
    for (int iy = 0; iy < L.my; iy++)
        for (int ix = 0; ix < L.mx; ix++) {
            const int ii = ix + iy * L.mx;
            if (!(L.pn[ii] > 0.0)) continue;
            const double xp[2] = {L.xc1 + ix * L.dx, neg * (L.yc1 + iy * L.dy)};
            stres1_pcwcns(L.dx, L.dy, L.gg[ia], v, vnu, xw, xp);
            const double p[3] = {L.px[ii], L.py[ii], L.pn[ii]};
            for (int j = 0; j < 3; j++)
                for (int k = 0; k < 4; k++)
                    for (int i = 0; i < 3; i++) {
                        const int fi = (i == 0) ? neg : 1;
                        vr[j][k] += fi * p[i] * (v[i][j][k] + L.poiss[ia] * vnu[i][j][k]);
                    }
        }
    return sstres_derived(L.gg[ia], L.poiss[ia], neg, vr);
}

// sstres_inflcf + sstres_fft, m_subsurf.f90:1097-1408: the field at depth zw at every element
// centre, from influence coefficients of a unit element at all offsets (the quarter ix, iy <= 0
// computed, the rest by symmetry) and the FFT convolution of the solve path (ga = 1)
inline void sstres_fft_depth(const SubsLoad &L, double zw, SubsPoint *out) {
    const int mx = L.mx, my = L.my, npot = mx * my;
    const int ia = (zw >= 0.0) ? 0 : 1, neg = (zw >= 0.0) ? 1 : -1;
    Inflcf ck[4];
    for (int k = 0; k < 4; k++) {
        ck[k].alloc(mx, my, L.dx, L.dy);
        ck[k].ga = 1.0; ck[k].ga_inv = 1.0; ck[k].nt_cpl = true;
    }
    const int nx = mx, ny = my;                    // offsets of the full grid (ixl = 1, ixh = mx)
    double v[3][3][4], vnu[3][3][4];
    for (int iy = -ny; iy <= 0; iy++)
        for (int ix = -nx; ix <= 0; ix++) {
            const double xp[2] = {0.0, 0.0};
            const double xw[3] = {(double)(float)ix * L.dx, neg * (double)(float)iy * L.dy, neg * zw};
            stres1_pcwcns(L.dx, L.dy, L.gg[ia], v, vnu, xw, xp);
            for (int k = 0; k < 4; k++)
                for (int i = 0; i < 3; i++)
                    for (int j = 0; j < 3; j++)
                        ck[k].at(ix, iy, j + 1, i + 1) = v[i][j][k] + L.poiss[ia] * vnu[i][j][k];
        }
    for (int k = 0; k < 4; k++)
        for (int ik = 1; ik <= 3; ik++)
            for (int jk = 1; jk <= 3; jk++) {
                const int f = (k == 1 ? -1 : 1) * (ik == 1 ? -1 : 1) * (jk == 1 ? -1 : 1);
                for (int iy = -ny; iy <= 0; iy++)
                    for (int ix = 1; ix <= nx - 1; ix++) ck[k].at(ix, iy, jk, ik) = f * ck[k].at(-ix, iy, jk, ik);
            }
    for (int k = 0; k < 4; k++)
        for (int ik = 1; ik <= 3; ik++)
            for (int jk = 1; jk <= 3; jk++) {
                const int f = (k == 2 ? -1 : 1) * (ik == 2 ? -1 : 1) * (jk == 2 ? -1 : 1);
                for (int iy = 1; iy <= ny - 1; iy++)
                    for (int ix = -nx; ix <= nx - 1; ix++) ck[k].at(ix, iy, jk, ik) = f * ck[k].at(ix, -iy, jk, ik);
            }
    // z < 0: px negated.  The reference negates the caller's px in place at every such depth,
    // so that its sign alternates from one depth to the next; here it is negated once per depth.
    GF3 ps, u;
    ps.init(npot); u.init(npot);
    for (int ii = 0; ii < npot; ii++) {
        ps.vx(ii) = (ia == 1 ? -1.0 : 1.0) * L.px[ii];
        ps.vy(ii) = L.py[ii];
        ps.vn(ii) = L.pn[ii];
    }
    Eldiv igs; igs.init(mx, my);
    for (int ii = 0; ii < npot; ii++) igs.el[ii] = (L.pn[ii] > 0.0) ? Adhes : Exter;
    areas(igs);
    std::vector<double> vr((size_t)npot * 12, 0.0);            // vr[ii][ik][k]
    for (int k = 0; k < 4; k++) {
        vecaijpj(igs, AllElm, u, ikALL, ps, igs, -3, ck[k], mx, my);
        for (int ik = 0; ik < 3; ik++)
            for (int ii = 0; ii < npot; ii++) vr[(size_t)ii * 12 + ik * 4 + k] = u.c[ik][ii];
    }
    for (int ii = 0; ii < npot; ii++) {
        double w[3][4];
        for (int ik = 0; ik < 3; ik++)
            for (int k = 0; k < 4; k++) w[ik][k] = vr[(size_t)ii * 12 + ik * 4 + k];
        out[ii] = sstres_derived(L.gg[ia], L.poiss[ia], neg, w);
    }
}

} // namespace orc
