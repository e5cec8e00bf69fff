// CPU ORACLE -- test infrastructure only (see contact_oracle.h).
//
// Core data structures of the oracle: uniform grid, element division, 3-component
// grid functions, influence-coefficient matrices with their FFT cache, and the
// masked BLAS-1 operations of src/m_gridfunc.f90.  Index convention: element
// ii = (ix-1) + (iy-1)*nx for the reference's 1-based (ix,iy).
#pragma once
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <map>
#include <vector>
#include <algorithm>

namespace orc {

typedef std::complex<double> cplx;

// element-division codes, src/m_gridfunc.f90:29-37
constexpr int AllElm = -9, AllInt = -8, AllExt = -7;
constexpr int Exter = 0, Adhes = 1, Slip = 2, Plast = 3;
// direction codes, src/m_globals.f90:42-43
constexpr int ikX = 1, ikY = 2, ikZ = 3, ikTANG = -2, ikALL = -3;
constexpr double tiny_ = 1e-20;             // src/m_globals.f90:36
static const double pi = 4.0 * std::atan(1.0);

// solver ids, src/m_hierarch_data.f90:113-116
constexpr int isolv_normcg = 1, isolv_tangcg = 2, isolv_cnvxgs = 3, isolv_stdygs = 4, isolv_gdstdy = 7;

inline void ikrange(int ik, int &k0, int &k1) {   // gf3_ikrange, m_gridfunc.f90:715-737
    if (ik == ikALL) { k0 = 1; k1 = 3; }
    else if (ik == ikTANG) { k0 = 1; k1 = 2; }
    else if (ik >= 1 && ik <= 3) { k0 = k1 = ik; }
    else { k0 = 1; k1 = 0; }
}

inline void igsrange(int iigs, int &g0, int &g1) { // IgsRange, m_aijpj.f90:68-95
    if (iigs == AllElm) { g0 = Exter; g1 = Plast; }
    else if (iigs == AllExt) { g0 = Exter; g1 = Exter; }
    else if (iigs == AllInt) { g0 = Adhes; g1 = Plast; }
    else if (iigs >= Exter && iigs <= Plast) { g0 = g1 = iigs; }
    else { g0 = Adhes; g1 = Exter; }
}

struct Grid {                                      // grid_create_uniform, m_grids.f90:559-703
    int nx = 1, ny = 1, n = 1;
    double dx = 1, dy = 1, dxdy = 1, x0 = 0, y0 = 0;
    std::vector<double> x, y;
    void create(int nx_, double x0_, double dx_, int ny_, double y0_, double dy_) {
        nx = nx_; ny = ny_; n = nx * ny; dx = dx_; dy = dy_; dxdy = dx * dy; x0 = x0_; y0 = y0_;
        x.assign(n, 0.0); y.assign(n, 0.0);
        for (int iy = 1; iy <= ny; iy++) {
            double yy = y0 + (iy - 1) * dy;
            for (int ix = 1; ix <= nx; ix++) {
                int ii = (ix - 1) + (iy - 1) * nx;
                x[ii] = x0 + (ix - 1) * dx;
                y[ii] = yy;
            }
        }
    }
};

struct Eldiv {                                     // t_eldiv, m_gridfunc.f90:117-139
    std::vector<int> el, row1st, rowlst;           // row1st/rowlst hold 1-based ix
    int ixmin = 1, ixmax = 1, iymin = 1, iymax = 1;
    int nx = 1, ny = 1;
    void init(int nx_, int ny_) {
        nx = nx_; ny = ny_;
        el.assign((size_t)nx * ny, Exter);
        row1st.assign(ny, nx); rowlst.assign(ny, 0);
    }
};

// Areas, m_gridfunc.f90:582-637
inline void areas(Eldiv &e) {
    int nx = e.nx, ny = e.ny;
    e.ixmin = nx; e.ixmax = 1; e.iymin = ny; e.iymax = 1;
    for (int iy = 1; iy <= ny; iy++) {
        int i0 = (iy - 1) * nx;
        int first = 1;
        while (e.el[(first - 1) + i0] <= Exter && first != nx) first++;
        int last = 0;
        for (int ix = first; ix <= nx; ix++)
            if (e.el[(ix - 1) + i0] >= Adhes) last = ix;
        e.row1st[iy - 1] = first;
        e.rowlst[iy - 1] = last;
        if (first <= last) {
            e.ixmin = std::min(e.ixmin, first); e.ixmax = std::max(e.ixmax, last);
            e.iymin = std::min(e.iymin, iy);    e.iymax = std::max(e.iymax, iy);
        }
    }
}

inline void eldiv_count(const Eldiv &e, int &nadh, int &nslip, int &nplast, int &nexter) {
    nadh = nslip = nplast = nexter = 0;                 // m_gridfunc.f90:406-433
    for (int v : e.el) {
        if (v == Adhes) nadh++; else if (v == Slip) nslip++; else if (v == Plast) nplast++; else nexter++;
    }
}

// eldiv_count_atbnd, m_gridfunc.f90:437-490 (rowcol = 0)
inline int eldiv_count_atbnd(const Eldiv &e) {
    int nx = e.nx, ny = e.ny, icount = 0;
    int iystep = (nx >= 3) ? 1 : std::max(1, ny - 1);
    for (int iy = 1; iy <= ny; iy += iystep) {
        int ixstep = (ny >= 3 && (iy == 1 || iy == ny)) ? 1 : std::max(1, nx - 1);
        for (int ix = 1; ix <= nx; ix += ixstep)
            if (e.el[(ix - 1) + (iy - 1) * nx] >= Adhes) icount++;
    }
    return icount;
}

// three-column grid function, t_gridfnc3 (m_gridfunc.f90:157-181); column ik-1 holds direction ik
struct GF3 {
    std::vector<double> c[3];
    int n = 0;
    void init(int n_) { n = n_; for (auto &v : c) v.assign(n, 0.0); }
    double *col(int ik) { return c[ik - 1].data(); }
    const double *col(int ik) const { return c[ik - 1].data(); }
    double &vx(int i) { return c[0][i]; }
    double &vy(int i) { return c[1][i]; }
    double &vn(int i) { return c[2][i]; }
};

// masked BLAS-1, m_gridfunc.f90:936-1510.  'ed' is the element division the grid
// function carries (f%eldiv in the reference).
inline void gf_set(int iigs, double val, GF3 &f, int ik, const Eldiv &ed) {
    int k0, k1; ikrange(ik, k0, k1);
    for (int k = k0; k <= k1; k++) {
        double *v = f.col(k);
        for (int i = 0; i < f.n; i++)
            if (iigs == AllElm || ed.el[i] >= Adhes) v[i] = val;
    }
}
inline void gf_copy(int iigs, const GF3 &a, GF3 &b, int ik, const Eldiv &ed) {
    int k0, k1; ikrange(ik, k0, k1);
    for (int k = k0; k <= k1; k++) {
        const double *s = a.col(k); double *d = b.col(k);
        for (int i = 0; i < a.n; i++)
            if (iigs == AllElm || ed.el[i] >= Adhes) d[i] = s[i];
    }
}
inline void gf_scal(int iigs, double s, GF3 &f, int ik, const Eldiv &ed) {
    int k0, k1; ikrange(ik, k0, k1);
    for (int k = k0; k <= k1; k++) {
        double *v = f.col(k);
        for (int i = 0; i < f.n; i++)
            if (iigs == AllElm || ed.el[i] >= Adhes) v[i] = s * v[i];
    }
}
// f2 := f2 + a f1 ; AllInt mask from f2's element division
inline void gf_axpy(int iigs, double a, const GF3 &f1, GF3 &f2, int ik, const Eldiv &ed) {
    int k0, k1; ikrange(ik, k0, k1);
    for (int k = k0; k <= k1; k++) {
        const double *s = f1.col(k); double *d = f2.col(k);
        for (int i = 0; i < f1.n; i++)
            if (iigs == AllElm || ed.el[i] >= Adhes) d[i] = d[i] + a * s[i];
    }
}
inline double gf_sum(int iigs, const GF3 &f, int ik, const Eldiv &ed) {
    int k0, k1; ikrange(ik, k0, k1);
    double s = 0;
    for (int k = k0; k <= k1; k++) {
        const double *v = f.col(k);
        for (int i = 0; i < f.n; i++)
            if (iigs == AllElm || ed.el[i] >= Adhes) s += v[i];
    }
    return s;
}
inline void gf_proj_avg(int iigs, GF3 &f, int ik, const Eldiv &ed) {
    int k0, k1; ikrange(ik, k0, k1);
    for (int k = k0; k <= k1; k++) {
        double *v = f.col(k);
        if (iigs == AllElm) {
            double s = 0; for (int i = 0; i < f.n; i++) s += v[i];
            double avg = s / (double)f.n;
            for (int i = 0; i < f.n; i++) v[i] -= avg;
        } else {
            double avg = 0; int nval = 0;
            for (int i = 0; i < f.n; i++) if (ed.el[i] >= Adhes) { avg += v[i]; nval++; }
            avg = avg / (double)std::max(1, nval);
            for (int i = 0; i < f.n; i++) if (ed.el[i] >= Adhes) v[i] -= avg;
        }
    }
}
// gf3_dot; mask taken from f1's element division
inline double gf_dot(int iigs, const GF3 &a, const GF3 &b, int ik, const Eldiv &ed) {
    int k0, k1; ikrange(ik, k0, k1);
    double s = 0;
    for (int k = k0; k <= k1; k++) {
        const double *x = a.col(k), *y = b.col(k);
        for (int i = 0; i < a.n; i++) {
            bool on = (iigs == AllElm) || (iigs == AllInt ? ed.el[i] >= Adhes : ed.el[i] == iigs);
            if (on) s += x[i] * y[i];
        }
    }
    return s;
}
inline double gf_nrm2(int iigs, const GF3 &f, int ik, const Eldiv &ed) {
    int k0, k1; ikrange(ik, k0, k1);
    double s = 0;
    for (int k = k0; k <= k1; k++) {
        const double *v = f.col(k);
        for (int i = 0; i < f.n; i++) if (iigs == AllElm || ed.el[i] >= Adhes) s += v[i] * v[i];
    }
    return std::sqrt(s);
}
inline double gf_rms(int iigs, const GF3 &f, int ik, const Eldiv &ed) {
    int k0, k1; ikrange(ik, k0, k1);
    double s = 0; int cnt = 0;
    for (int k = k0; k <= k1; k++) {
        const double *v = f.col(k);
        for (int i = 0; i < f.n; i++) if (iigs == AllElm || ed.el[i] >= Adhes) { s += v[i] * v[i]; cnt++; }
    }
    return std::sqrt(s / std::max(1, cnt));
}
inline double gf_min(int iigs, const GF3 &f, int ik, const Eldiv &ed) {
    double m = 1e20; const double *v = f.col(ik);
    for (int i = 0; i < f.n; i++) if ((iigs == AllElm || ed.el[i] >= Adhes) && v[i] < m) m = v[i];
    return m;
}
inline double gf_max(int iigs, const GF3 &f, int ik, const Eldiv &ed) {
    double m = -1e20; const double *v = f.col(ik);
    for (int i = 0; i < f.n; i++) if ((iigs == AllElm || ed.el[i] >= Adhes) && v[i] > m) m = v[i];
    return m;
}

// ---------------------------------------------------------------------------------------------
// Mixed-radix complex FFT (own implementation; the reference links Intel MKL DFTI).
// Recursive decimation in time with a generic radix-p butterfly; unnormalised.
// ---------------------------------------------------------------------------------------------
struct FFTPlan {
    int n = 0;
    std::vector<int> fac;
    std::vector<cplx> w;    // w[j] = exp(-2 pi i j / n)
};

inline const FFTPlan &fft_plan(int n) {
    static thread_local std::map<int, FFTPlan> cache;
    auto it = cache.find(n);
    if (it != cache.end()) return it->second;
    FFTPlan p; p.n = n;
    int m = n;
    for (int f : {4, 2, 3, 5, 7}) while (m % f == 0) { p.fac.push_back(f); m /= f; }
    for (int f = 11; m > 1; f += 2) while (m % f == 0) { p.fac.push_back(f); m /= f; }
    p.w.resize(n);
    for (int j = 0; j < n; j++) {
        double a = -2.0 * pi * (double)j / (double)n;
        p.w[j] = cplx(std::cos(a), std::sin(a));
    }
    return cache.emplace(n, std::move(p)).first->second;
}

inline void fft_rec(const cplx *in, int stride, cplx *out, int n, const int *fac,
                    const FFTPlan &pl, int wstep, bool inv, cplx *tmp) {
    if (n == 1) { out[0] = in[0]; return; }
    int p = fac[0], m = n / p;
    for (int r = 0; r < p; r++)
        fft_rec(in + (size_t)r * stride, stride * p, out + (size_t)r * m, m, fac + 1, pl, wstep * p, inv, tmp);
    // combine: X[k + q m] = sum_r W_n^{r (k + q m)} Y_r[k]
    for (int k = 0; k < m; k++) {
        for (int q = 0; q < p; q++) {
            cplx s(0, 0);
            for (int r = 0; r < p; r++) {
                long e = ((long)r * (k + (long)q * m)) % n;
                cplx w = pl.w[(size_t)e * wstep];
                if (inv) w = std::conj(w);
                s += w * out[(size_t)r * m + k];
            }
            tmp[k + q * m] = s;
        }
    }
    for (int j = 0; j < n; j++) out[j] = tmp[j];
}

inline void fft1d(cplx *a, int n, bool inv) {
    const FFTPlan &pl = fft_plan(n);
    std::vector<cplx> in(a, a + n), tmp(n);
    fft_rec(in.data(), 1, a, n, pl.fac.data(), pl, 1, inv, tmp.data());
}

#ifndef ORC_FAST_FFT
// 2-D transform of a (nx fastest, ny rows)
inline void fft2d(std::vector<cplx> &a, int nx, int ny, bool inv) {
    for (int iy = 0; iy < ny; iy++) fft1d(a.data() + (size_t)iy * nx, nx, inv);
    std::vector<cplx> col(ny);
    for (int ix = 0; ix < nx; ix++) {
        for (int iy = 0; iy < ny; iy++) col[iy] = a[ix + (size_t)iy * nx];
        fft1d(col.data(), ny, inv);
        for (int iy = 0; iy < ny; iy++) a[ix + (size_t)iy * nx] = col[iy];
    }
}
#else
// ---------------------------------------------------------------------------------------------
// Baseline build (-DORC_FAST_FFT): the same transforms by an iterative Stockham autosort FFT
// (Stockham's self-sorting formulation, as in Van Loan, "Computational Frameworks for the
// Fast Fourier Transform", 1992, sec. 1.7) with radix-4/2/3/5/7 butterflies, per-stage
// twiddle tables and rows and columns transformed in interleaved blocks, and the
// convolutions through real-input transforms (real_conv2d).  It stands in for the optimised
// FFT library the reference links, so that the timed CPU baseline is not slowed by the
// simple recursive FFT above; results agree with it to rounding.
// ---------------------------------------------------------------------------------------------
struct StockhamPlan {
    int n = 0;
    std::vector<int> rad;
    std::vector<std::vector<cplx>> tw;     // per stage: w^(r k), k < Ns, r < p, w = exp(-2 pi i / (Ns p))
    std::vector<std::vector<cplx>> roots;  // per stage of a radix above 5: exp(-2 pi i q / p), q < p
};

inline const StockhamPlan &stockham_plan(int n) {
    static thread_local std::map<int, StockhamPlan> cache;
    auto it = cache.find(n);
    if (it != cache.end()) return it->second;
    StockhamPlan p; p.n = n;
    int m = n;
    for (int f : {4, 2, 3, 5}) while (m % f == 0) { p.rad.push_back(f); m /= f; }
    for (int f = 7; m > 1; f += 2) while (m % f == 0) { p.rad.push_back(f); m /= f; }
    int ns = 1;
    for (int r : p.rad) {
        std::vector<cplx> t((size_t)ns * r);
        for (int k = 0; k < ns; k++)
            for (int q = 0; q < r; q++) {
                const double a = -2.0 * pi * (double)((long)q * k) / (double)((long)ns * r);
                t[(size_t)k * r + q] = cplx(std::cos(a), std::sin(a));
            }
        p.tw.push_back(std::move(t));
        std::vector<cplx> ro;
        if (r > 5)
            for (int q = 0; q < r; q++) {
                const double a = -2.0 * pi * (double)q / (double)r;
                ro.push_back(cplx(std::cos(a), std::sin(a)));
            }
        p.roots.push_back(std::move(ro));
        ns *= r;
    }
    return cache.emplace(n, std::move(p)).first->second;
}

// Butterflies of one Stockham stage: v[0..P-1] -> their length-P DFT (sg = -1 forward, +1
// inverse); radices above 5 by the direct sum with the roots exp(sg 2 pi i q / P)
template <int P>
inline void butterfly(cplx *v, double sg, const cplx *roots) {
    if constexpr (P == 2) {
        const cplx a = v[0], b = v[1];
        v[0] = a + b; v[1] = a - b;
    } else if constexpr (P == 4) {
        const cplx a0 = v[0] + v[2], a1 = v[0] - v[2], a2 = v[1] + v[3], a3 = v[1] - v[3];
        const cplx a3r(-sg * a3.imag(), sg * a3.real());     // a3 * (sg i)
        v[0] = a0 + a2; v[2] = a0 - a2; v[1] = a1 + a3r; v[3] = a1 - a3r;
    } else if constexpr (P == 3) {
        const double c1 = -0.5, s1 = sg * 0.86602540378443864676;
        const cplx a = v[0], b = v[1], c = v[2];
        const cplx t1 = b + c, t2 = a + c1 * t1;
        const cplx t3(-s1 * (b - c).imag(), s1 * (b - c).real());
        v[0] = a + t1; v[1] = t2 + t3; v[2] = t2 - t3;
    } else if constexpr (P == 5) {
        const double c1 = 0.30901699437494742410, c2 = -0.80901699437494742410;
        const double s1 = sg * 0.95105651629515357212, s2 = sg * 0.58778525229247312917;
        const cplx a = v[0], b1 = v[1] + v[4], b2 = v[2] + v[3], d1 = v[1] - v[4], d2 = v[2] - v[3];
        const cplx t1 = a + c1 * b1 + c2 * b2, t2 = a + c2 * b1 + c1 * b2;
        const cplx u1 = s1 * d1 + s2 * d2, u2 = s2 * d1 - s1 * d2;
        const cplx i1(-u1.imag(), u1.real()), i2(-u2.imag(), u2.real());
        v[0] = a + b1 + b2; v[1] = t1 + i1; v[4] = t1 - i1; v[2] = t2 + i2; v[3] = t2 - i2;
    } else {
        cplx out[P];
        for (int q = 0; q < P; q++) {
            cplx acc = v[0];
            for (int r = 1; r < P; r++) acc += v[r] * roots[(size_t)((long)r * q % P)];
            out[q] = acc;
        }
        for (int q = 0; q < P; q++) v[q] = out[q];
    }
}

// one Stockham stage of radix P over 'cnt' interleaved transforms (element e of transform t
// at x[e * cnt + t]), the transforms innermost so that the loop over them vectorises
template <int P>
inline void stockham_stage_r(const cplx *x, cplx *y, int n, int ns, const cplx *tw, const cplx *roots, bool inv,
                             int cnt) {
    const int nb = n / P;
    const double sg = inv ? 1.0 : -1.0;
    cplx ro[P > 5 ? P : 1];
    if constexpr (P > 5)
        for (int q = 0; q < P; q++) ro[q] = inv ? std::conj(roots[q]) : roots[q];
    for (int j = 0; j < nb; j++) {
        const int k = j % ns;
        const int o = (j / ns) * ns * P + k;
        cplx w[P];
        for (int r = 0; r < P; r++) w[r] = inv ? std::conj(tw[(size_t)k * P + r]) : tw[(size_t)k * P + r];
        const cplx *xr[P];
        cplx *yr[P];
        for (int r = 0; r < P; r++) {
            xr[r] = x + (size_t)(j + r * nb) * cnt;
            yr[r] = y + (size_t)(o + r * ns) * cnt;
        }
        for (int t = 0; t < cnt; t++) {
            cplx v[P];
            v[0] = xr[0][t];
            for (int r = 1; r < P; r++) v[r] = xr[r][t] * w[r];
            butterfly<P>(v, sg, ro);
            for (int r = 0; r < P; r++) yr[r][t] = v[r];
        }
    }
}

inline void stockham_stage(const cplx *x, cplx *y, int n, int ns, int p, const cplx *tw, const cplx *roots,
                           bool inv, int cnt) {
    switch (p) {
    case 2: stockham_stage_r<2>(x, y, n, ns, tw, roots, inv, cnt); break;
    case 3: stockham_stage_r<3>(x, y, n, ns, tw, roots, inv, cnt); break;
    case 4: stockham_stage_r<4>(x, y, n, ns, tw, roots, inv, cnt); break;
    case 5: stockham_stage_r<5>(x, y, n, ns, tw, roots, inv, cnt); break;
    case 7: stockham_stage_r<7>(x, y, n, ns, tw, roots, inv, cnt); break;
    default: {
        // other odd primes (not produced by opt_fft_size): the direct sum, one element at a time
        const int nb = n / p;
        std::vector<cplx> v(p), out(p);
        for (int j = 0; j < nb; j++) {
            const int k = j % ns;
            const int o = (j / ns) * ns * p + k;
            for (int t = 0; t < cnt; t++) {
                for (int r = 0; r < p; r++) {
                    cplx a = x[(size_t)(j + r * nb) * cnt + t];
                    const cplx wr = tw[(size_t)k * p + r];
                    v[r] = a * (inv ? std::conj(wr) : wr);
                }
                for (int q = 0; q < p; q++) {
                    cplx acc = v[0];
                    for (int r = 1; r < p; r++) {
                        const cplx w = roots[(size_t)((long)r * q % p)];
                        acc += v[r] * (inv ? std::conj(w) : w);
                    }
                    out[q] = acc;
                }
                for (int r = 0; r < p; r++) y[(size_t)(o + r * ns) * cnt + t] = out[r];
            }
        }
    }
    }
}

// cnt interleaved transforms of length n in a (element e of transform t at a[e * cnt + t])
inline void stockham_many(cplx *a, int n, int cnt, bool inv, std::vector<cplx> &scratch) {
    const StockhamPlan &pl = stockham_plan(n);
    if (scratch.size() < (size_t)n * cnt) scratch.resize((size_t)n * cnt);   // grows only
    cplx *src = a, *dst = scratch.data();
    int ns = 1;
    for (size_t s = 0; s < pl.rad.size(); s++) {
        stockham_stage(src, dst, n, ns, pl.rad[s], pl.tw[s].data(), pl.roots[s].data(), inv, cnt);
        ns *= pl.rad[s];
        std::swap(src, dst);
    }
    if (src != a) std::copy(src, src + (size_t)n * cnt, a);
}

// 2-D transform of a (nx fastest, ny rows): rows and columns in interleaved blocks of 16
inline void fft2d(std::vector<cplx> &a, int nx, int ny, bool inv) {
    thread_local std::vector<cplx> scratch, blk;
    const int B = 16;
    for (int iy0 = 0; iy0 < ny; iy0 += B) {
        const int w = std::min(B, ny - iy0);
        if (blk.size() < (size_t)nx * w) blk.resize((size_t)nx * w);
        for (int t = 0; t < w; t++)
            for (int e = 0; e < nx; e++) blk[(size_t)e * w + t] = a[(size_t)(iy0 + t) * nx + e];
        stockham_many(blk.data(), nx, w, inv, scratch);
        for (int t = 0; t < w; t++)
            for (int e = 0; e < nx; e++) a[(size_t)(iy0 + t) * nx + e] = blk[(size_t)e * w + t];
    }
    for (int ix0 = 0; ix0 < nx; ix0 += B) {
        const int w = std::min(B, nx - ix0);
        if (blk.size() < (size_t)ny * w) blk.resize((size_t)ny * w);
        for (int iy = 0; iy < ny; iy++)
            for (int t = 0; t < w; t++) blk[(size_t)iy * w + t] = a[(size_t)iy * nx + ix0 + t];
        stockham_many(blk.data(), ny, w, inv, scratch);
        for (int iy = 0; iy < ny; iy++)
            for (int t = 0; t < w; t++) a[(size_t)iy * nx + ix0 + t] = blk[(size_t)iy * w + t];
    }
}

// Circular convolution of a real nx x ny grid (nx, ny even) with the kernel whose full
// spectrum is cf, by real-input transforms as the reference's FFT library computes it:
// two real rows packed into one complex row transform, then the nx/2+1 columns that
// Hermitian symmetry leaves, the product with the spectrum, and the way back.  out =
// IFFT(cf .* FFT(in)) without the 1/(nx ny) scaling, as fft2d's inverse.
inline void real_conv2d(const double *in, const cplx *cf, int nx, int ny, double *out) {
    thread_local std::vector<cplx> H, blk, scratch;
    const int hx = nx / 2 + 1, B = 8;
    if (H.size() < (size_t)ny * hx) H.resize((size_t)ny * hx);
    const cplx mhalf_i(0.0, -0.5);
    for (int q0 = 0; q0 < ny / 2; q0 += B) {
        const int w = std::min(B, ny / 2 - q0);
        if (blk.size() < (size_t)nx * w) blk.resize((size_t)nx * w);
        for (int t = 0; t < w; t++) {
            const double *r0 = in + (size_t)(2 * (q0 + t)) * nx, *r1 = r0 + nx;
            for (int e = 0; e < nx; e++) blk[(size_t)e * w + t] = cplx(r0[e], r1[e]);
        }
        stockham_many(blk.data(), nx, w, false, scratch);
        for (int t = 0; t < w; t++) {
            cplx *h0 = H.data() + (size_t)(2 * (q0 + t)) * hx, *h1 = h0 + hx;
            for (int k = 0; k < hx; k++) {
                const cplx zk = blk[(size_t)k * w + t], zn = std::conj(blk[(size_t)((nx - k) % nx) * w + t]);
                h0[k] = 0.5 * (zk + zn);
                h1[k] = mhalf_i * (zk - zn);
            }
        }
    }
    const int BC = 16;
    for (int k0 = 0; k0 < hx; k0 += BC) {
        const int w = std::min(BC, hx - k0);
        if (blk.size() < (size_t)ny * w) blk.resize((size_t)ny * w);
        for (int iy = 0; iy < ny; iy++)
            for (int t = 0; t < w; t++) blk[(size_t)iy * w + t] = H[(size_t)iy * hx + k0 + t];
        stockham_many(blk.data(), ny, w, false, scratch);
        for (int iy = 0; iy < ny; iy++)
            for (int t = 0; t < w; t++) blk[(size_t)iy * w + t] *= cf[(size_t)(k0 + t) + (size_t)iy * nx];
        stockham_many(blk.data(), ny, w, true, scratch);
        for (int iy = 0; iy < ny; iy++)
            for (int t = 0; t < w; t++) H[(size_t)iy * hx + k0 + t] = blk[(size_t)iy * w + t];
    }
    const cplx iu(0.0, 1.0);
    for (int q0 = 0; q0 < ny / 2; q0 += B) {
        const int w = std::min(B, ny / 2 - q0);
        if (blk.size() < (size_t)nx * w) blk.resize((size_t)nx * w);
        for (int t = 0; t < w; t++) {
            const cplx *h0 = H.data() + (size_t)(2 * (q0 + t)) * hx, *h1 = h0 + hx;
            for (int k = 0; k < hx; k++) blk[(size_t)k * w + t] = h0[k] + iu * h1[k];
            for (int k = hx; k < nx; k++) blk[(size_t)k * w + t] = std::conj(h0[nx - k]) + iu * std::conj(h1[nx - k]);
        }
        stockham_many(blk.data(), nx, w, true, scratch);
        for (int t = 0; t < w; t++) {
            double *r0 = out + (size_t)(2 * (q0 + t)) * nx, *r1 = r0 + nx;
            for (int e = 0; e < nx; e++) {
                r0[e] = blk[(size_t)e * w + t].real();
                r1[e] = blk[(size_t)e * w + t].imag();
            }
        }
    }
}
#endif

// opt_fft_size, m_aijpj.f90:1022-1119: a 2^a 3^b 5^c 7^d >= n found greedily, starting from the next
// power of two and trading factors while the product stays >= n (not always the smallest such number)
inline int opt_fft_size(int fft_size) {
    static const int kpat[9][8] = {
        {-2, 1, 0, 0, 0, 4, 3, 3},   {-5, 3, 0, 0, 0, 32, 27, 3},  {-1, -1, 1, 0, 0, 6, 5, 5},
        {-4, 1, 1, 0, 0, 16, 15, 5}, {0, -3, 2, 0, 0, 27, 25, 5},  {-3, 0, 0, 1, 0, 8, 7, 7},
        {1, -1, -1, 1, 0, 15, 14, 7}, {-1, 2, -1, 0, 0, 10, 9, 5}, {-2, -1, 0, 0, 1, 12, 11, 11}};
    const int use_fac = 7;
    int k2 = (int)std::ceil(std::log(1.0 * fft_size) / std::log(2.0));
    long prod = 1L << k2;
    int kf[5] = {k2, 0, 0, 0, 0};
    bool changed = true;
    while (changed) {
        changed = false;
        for (int ip = 0; ip < 9; ip++) {
            const int *kp = kpat[ip];
            if (kp[5] > 0 && kp[7] <= use_fac) {
                while (true) {
                    bool ok = true;
                    for (int f = 0; f < 5; f++) if (kf[f] + kp[f] < 0) ok = false;
                    if (!(ok && (long)kp[6] * prod >= (long)kp[5] * fft_size)) break;
                    for (int f = 0; f < 5; f++) kf[f] += kp[f];
                    prod = (long)kp[6] * prod / kp[5];
                    changed = true;
                }
            }
        }
    }
    return (int)prod;
}

// ---------------------------------------------------------------------------------------------
// influence-coefficient matrix, t_inflcf (m_inflcf.f90:49-106)
// ---------------------------------------------------------------------------------------------
struct Inflcf {
    int cf_mx = 0, cf_my = 0;
    double dx = 0, dy = 0, dq = 0;
    bool nt_cpl = true;
    double ga = 1, ga_inv = 1;
    // interfacial layer of M=4 (inflcf_mater, m_hierarch_data.f90:1557-1570): flexibility
    // laythk / gg3 of px on ux and py on uy
    bool use_3bl = false;
    double flx_3bl = 0;
    std::vector<double> cf[3][3];                 // (2cf_mx)*(2cf_my), ix fastest
    int fft_mx = -1, fft_my = -1;
    bool fft_ok[3][3] = {};
    std::vector<cplx> fft_cf[3][3];               // full 2fft_mx*2fft_my spectrum

    bool defined() const { return cf_mx >= 1 && cf_my >= 1 && !cf[0][0].empty(); }
    void alloc(int mx, int my, double dx_, double dy_) {   // inflcf_new_mxmy, m_inflcf.f90:147-219
        cf_mx = mx; cf_my = my; dx = dx_; dy = dy_; dq = dx_;
        for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) cf[i][j].assign((size_t)4 * mx * my, 0.0);
        nt_cpl = true;
        fft_mx = 2 * mx; fft_my = 2 * my;
        for (auto &r : fft_ok) for (bool &b : r) b = false;
        for (auto &r : fft_cf) for (auto &v : r) v.clear();
    }
    double &at(int ix, int iy, int ik, int jk) {
        return cf[ik - 1][jk - 1][(size_t)(ix + cf_mx) + (size_t)(iy + cf_my) * 2 * cf_mx];
    }
    double at(int ix, int iy, int ik, int jk) const {
        return cf[ik - 1][jk - 1][(size_t)(ix + cf_mx) + (size_t)(iy + cf_my) * 2 * cf_mx];
    }
    void invalidate_fft() { for (auto &r : fft_ok) for (bool &b : r) b = false; }
};

} // namespace orc
