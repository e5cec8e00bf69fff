// Subsurface elastic field of the surface tractions on the GPU (m_subsurf.f90, module 3): the
// displacements and displacement gradients below a uniformly loaded rectangle (stres1_pcwcns,
// m_subsurf.f90:1633-1852, after Kalker, "Numerical calculation of the elastic field in a
// half-space", Comm. Appl. Num. Meth. 2, 1986, 401-410), summed over the loaded elements, and
// the stresses, invariants and principal stresses derived from them (sstres_derived,
// :1519-1629).  Piecewise-constant tractions (C = 2).
//
// Two forms, as the reference:
//   - arbitrary points (block type 9, sstres :1412-1515): one warp per point sums the field
//     of every loaded element;
//   - element centres at a depth (block types 1-7, sstres_inflcf + sstres_fft :1097-1408): the
//     influence coefficients of one element at all grid offsets are tabulated once per depth
//     (the quarter ix, iy <= 0 evaluated, the rest by the kernel's symmetries), then one warp
//     per selected element centre sums table x tractions over the loaded elements.  The
//     reference convolves the same table by FFT; the direct sum needs no spectra of the 36
//     blocks and keeps the whole depth in one pass.
#include <cuda_runtime.h>
#include "engine_api.h"

namespace cgb {

struct SubsDev {
    int mx, my;
    double dx, dy, xc1, yc1;
    const double *pn, *px, *py;
    double gg[2], poiss[2];
};

// One corner (jx, jy = +-1) of the dx x dy element centred at xp, seen from xw (xw[2] >= 0):
// its signed share of the displacements v[i][j][0] in direction j and their gradients
// v[i][j][k] (d/dx_k) due to a unit traction in direction i, added to v; vnu collects the
// parts proportional to Poisson's ratio.  The terms and their order of summation follow
// m_subsurf.f90:1633-1852; the four corners together, divided by 4 pi gg, give the field.
__device__ __noinline__ void stres1_corner(int jx, int jy, double dx, double dy, double v[3][3][4],
                                           double vnu[3][3][4], const double xw[3], const double xp[2]) {
    const double epsrel = 5e-7;
    const int sgn[3] = {-1, -1, 1};
    const int nxt[3] = {1, 2, 0};
    const double y[3] = {xp[0] + jx * dx / 2.0 - xw[0], xp[1] + jy * dy / 2.0 - xw[1], xw[2]};
    const double w = fmax(1e-12, sqrt(y[0] * y[0] + y[1] * y[1] + y[2] * y[2]));
    // components moved away from zero to at least epsrel w (with their sign), so that the
    // logarithms and quotients below stay finite on the element's edges
    const double epsy = epsrel * w;
    double ye[3];
    for (int i = 0; i < 3; i++) ye[i] = (y[i] >= 0.0) ? fmax(epsy, y[i]) : fmin(-epsy, y[i]);
    const double we = fmax(1e-12, sqrt(ye[0] * ye[0] + ye[1] * ye[1] + ye[2] * ye[2]));
    double al[3], at[3], wm[4];
    wm[0] = we;
    for (int k = 0; k < 3; k++) {
        al[k] = log(y[k] + we);
        at[k] = atan((y[nxt[k]] + y[nxt[nxt[k]]] + w) / ye[k]);
        wm[k + 1] = sgn[k] * y[k] / we;
    }
    double a[3][3][4], t[3][3][4];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            a[i][j][0] = y[i] * al[j];
            t[i][j][0] = y[i] * at[j];
            for (int k = 0; k < 3; k++) {
                const double dik = i == k ? 1.0 : 0.0, djk = j == k ? 1.0 : 0.0;
                a[i][j][k + 1] = sgn[k] * (dik * al[j] + y[i] * (djk * w + y[k]) / (we * (y[j] + we)));
                t[i][j][k + 1] = sgn[k] * (dik * at[j] +
                                           y[i] * (y[j] * (y[k] + w) - djk * w * (y[0] + y[1] + y[2] + w)) /
                                               (2 * we * (y[nxt[j]] + we) * (y[nxt[nxt[j]]] + we)));
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

// Displacements v[i][j][0] in direction j and their gradients v[i][j][k] (d/dx_k) at xw due to a
// unit traction in direction i on the dx x dy element centred at xp; vnu holds the parts
// proportional to Poisson's ratio.  xw[2] >= 0.  The four corners in the reference's order
// (m_subsurf.f90:1633-1852).
__device__ __noinline__ void stres1(double dx, double dy, double gg, double v[3][3][4], double vnu[3][3][4],
                                    const double xw[3], const double xp[2]) {
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            for (int k = 0; k < 4; k++) { v[i][j][k] = 0.0; vnu[i][j][k] = 0.0; }
    for (int jx = -1; jx <= 1; jx += 2)
        for (int jy = -1; jy <= 1; jy += 2) stres1_corner(jx, jy, dx, dy, v, vnu, xw, xp);
    const double f = 4.0 * 3.14159265358979323846 * gg;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            for (int k = 0; k < 4; k++) { v[i][j][k] /= f; vnu[i][j][k] /= f; }
}

// Eigenvalues of a symmetric 3x3 matrix, largest first, by the trigonometric solution of its
// characteristic cubic (O. K. Smith, Comm. ACM 4, 1961, 168)
__device__ inline void sym3_eig(const double s[3][3], double ev[3]) {
    const double pi = 3.14159265358979323846;
    const double p1 = s[0][1] * s[0][1] + s[0][2] * s[0][2] + s[1][2] * s[1][2];
    const double q = (s[0][0] + s[1][1] + s[2][2]) / 3.0;
    const double d0 = s[0][0] - q, d1 = s[1][1] - q, d2 = s[2][2] - q;
    const double p2 = d0 * d0 + d1 * d1 + d2 * d2 + 2.0 * p1;
    if (p2 <= 0.0) { ev[0] = ev[1] = ev[2] = q; return; }
    const double p = sqrt(p2 / 6.0);
    const double b00 = d0 / p, b11 = d1 / p, b22 = d2 / p, b01 = s[0][1] / p, b02 = s[0][2] / p, b12 = s[1][2] / p;
    double r = 0.5 * (b00 * (b11 * b22 - b12 * b12) - b01 * (b01 * b22 - b12 * b02) + b02 * (b01 * b12 - b11 * b02));
    r = fmax(-1.0, fmin(1.0, r));
    const double phi = acos(r) / 3.0;
    ev[0] = q + 2.0 * p * cos(phi);
    ev[2] = q + 2.0 * p * cos(phi + 2.0 * pi / 3.0);
    ev[1] = 3.0 * q - ev[0] - ev[2];
}

// sstres_derived, m_subsurf.f90:1519-1629: the components mirrored for body 2 (neg = -1),
// linearised strain, Hooke's law, invariants; values below gg 1e-15 set to zero.  out[18]:
// ux, uy, uz, sighyd, sigvm, sigtr, sigma1..3, sig[3][3] row by row.
__device__ void subs_derived(double gg, double poiss, int neg, double vr[3][4], double *out) {
    const double tolsml = 1e-15;
    for (int j = 0; j < 3; j++) {
        const int fj = (j == 1 || j == 2) ? neg : 1;
        for (int k = 0; k < 4; k++) {
            const int fk = (k == 2 || k == 3) ? neg : 1;
            vr[j][k] = fj * fk * vr[j][k];
        }
    }
    double u[3], er[3][3], sig[3][3], ev[3];
    for (int i = 0; i < 3; i++) u[i] = vr[i][0];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) er[i][j] = (vr[i][j + 1] + vr[j][i + 1]) / 2.0;
    const double dil = er[0][0] + er[1][1] + er[2][2];
    for (int j = 0; j < 3; j++)
        for (int i = 0; i < 3; i++) sig[i][j] = 2.0 * gg * er[i][j];
    for (int i = 0; i < 3; i++) sig[i][i] += 2.0 * gg * dil * poiss / fmax(1e-6, 1.0 - 2.0 * poiss);
    const double sigii = sig[0][0] + sig[1][1] + sig[2][2];
    double sijsij = -(1.0 / 3.0) * sigii * sigii;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) sijsij += sig[i][j] * sig[i][j];
    sijsij = 0.5 * sijsij;
    sym3_eig(sig, ev);
    for (int i = 0; i < 3; i++) out[i] = fabs(u[i]) < gg * tolsml ? 0.0 : u[i];
    out[3] = sigii / 3.0;
    out[4] = sqrt(3.0 * sijsij);
    out[5] = ev[0] - ev[2];
    for (int i = 0; i < 3; i++) out[6 + i] = ev[i];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) out[9 + 3 * i + j] = fabs(sig[i][j]) < gg * tolsml ? 0.0 : sig[i][j];
}

// the 12 sums of one output point, spread over the lanes of its warp, added up in a fixed
// order (shuffles down to lane 0)
__device__ inline void warp_sum12(double vr[3][4]) {
    for (int j = 0; j < 3; j++)
        for (int k = 0; k < 4; k++)
            for (int o = 16; o > 0; o >>= 1) vr[j][k] += __shfl_down_sync(0xffffffffu, vr[j][k], o);
}

// arbitrary points: the field of every element with positive pressure (sstres, :1412-1515).
// One warp per point; its lanes take every 32nd element of the grid, so that a few hundred
// points still fill the device.
__global__ void k_subs_points(SubsDev L, const double *xyz, int npts, double *out) {
    const int q = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (q >= npts) return;                     // whole warps: blockDim is a multiple of 32
    double xw[3] = {xyz[3 * q], xyz[3 * q + 1], xyz[3 * q + 2]};
    const int ia = (xw[2] >= 0.0) ? 0 : 1, neg = (xw[2] >= 0.0) ? 1 : -1;
    xw[2] = neg * xw[2];
    xw[1] = neg * xw[1];
    double vr[3][4] = {};
    double v[3][3][4], vnu[3][3][4];
    const int n = L.mx * L.my;
    for (int ii = lane; ii < n; ii += 32) {
        if (!(L.pn[ii] > 0.0)) continue;
        const int ix = ii % L.mx, iy = ii / L.mx;
        const double xp[2] = {L.xc1 + ix * L.dx, neg * (L.yc1 + iy * L.dy)};
        stres1(L.dx, L.dy, L.gg[ia], v, vnu, xw, xp);
        const double p[3] = {L.px[ii], L.py[ii], L.pn[ii]};
        for (int j = 0; j < 3; j++)
            for (int k = 0; k < 4; k++)
                for (int i = 0; i < 3; i++) {
                    const int fi = (i == 0) ? neg : 1;
                    vr[j][k] += fi * p[i] * (v[i][j][k] + L.poiss[ia] * vnu[i][j][k]);
                }
    }
    warp_sum12(vr);
    if (lane == 0) subs_derived(L.gg[ia], L.poiss[ia], neg, vr, out + (size_t)18 * q);
}

// influence coefficients of one element at depth zw (sstres_inflcf, :1261-1408): tab[b][off],
// block b = 9 k + 3 j + i (quantity k: displacement or d/dx_k, output direction j, traction
// direction i), offset (ix + mx) + (iy + my) 2mx for ix in [-mx, mx-1], iy in [-my, my-1].
// Four lanes per quarter offset ix, iy <= 0: lane c evaluates corner c of the element, the four
// shares are added across the lanes, and lane c writes the field with the signs of the
// kernel's symmetry in x and in y to mirror c of the offset (itself, in x, in y, in both).
__global__ void k_subs_table(SubsDev L, double zw, double *tab) {
    const int mx = L.mx, my = L.my, nq = (mx + 1) * (my + 1);
    const long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const int c = (int)(g & 3);
    // no early exit: every lane of the grid takes part in the shuffles (the grid holds whole
    // warps); lanes past the last offset compute the last one again and write nothing
    const bool live = (g >> 2) < nq;
    const int t = live ? (int)(g >> 2) : nq - 1;
    const int ix = -(t % (mx + 1)), iy = -(t / (mx + 1));
    const int ia = (zw >= 0.0) ? 0 : 1, neg = (zw >= 0.0) ? 1 : -1;
    const double xp[2] = {0.0, 0.0};
    const double xw[3] = {(double)(float)ix * L.dx, neg * (double)(float)iy * L.dy, neg * zw};
    double v[3][3][4], vnu[3][3][4];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            for (int k = 0; k < 4; k++) { v[i][j][k] = 0.0; vnu[i][j][k] = 0.0; }
    stres1_corner((c & 2) ? 1 : -1, (c & 1) ? 1 : -1, L.dx, L.dy, v, vnu, xw, xp);
    const double f = 4.0 * 3.14159265358979323846 * L.gg[ia];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            for (int k = 0; k < 4; k++) {
                double a = v[i][j][k], b = vnu[i][j][k];
                a += __shfl_xor_sync(0xffffffffu, a, 1);
                b += __shfl_xor_sync(0xffffffffu, b, 1);
                a += __shfl_xor_sync(0xffffffffu, a, 2);
                b += __shfl_xor_sync(0xffffffffu, b, 2);
                v[i][j][k] = a / f;
                vnu[i][j][k] = b / f;
            }
    const bool mirx = ix < 0 && -ix <= mx - 1, miry = iy < 0 && -iy <= my - 1;
    const bool wx = (c & 1) != 0, wy = (c & 2) != 0;
    if (!live || (wx && !mirx) || (wy && !miry)) return;
    const size_t bs = (size_t)4 * mx * my;
    const size_t o = (size_t)((wx ? -ix : ix) + mx) + (size_t)((wy ? -iy : iy) + my) * 2 * mx;
    for (int k = 0; k < 4; k++)
        for (int j = 0; j < 3; j++)
            for (int i = 0; i < 3; i++) {
                const double val = v[i][j][k] + L.poiss[ia] * vnu[i][j][k];
                const double fx = (k == 1 ? -1 : 1) * (j == 0 ? -1 : 1) * (i == 0 ? -1 : 1);
                const double fy = (k == 2 ? -1 : 1) * (j == 1 ? -1 : 1) * (i == 1 ? -1 : 1);
                double w = val;
                if (wx) w = fx * w;
                if (wy) w = fy * w;
                tab[(size_t)(9 * k + 3 * j + i) * bs + o] = w;
            }
}

// element centres (ixs[], iys[] 1-based) at depth zw: table x tractions summed over the
// elements (sstres_fft, :1097-1257, here as a direct sum); the x traction is negated for body
// 2.  One warp per centre; its lanes take every 32nd element, so consecutive lanes read
// consecutive table entries.
__global__ void k_subs_conv(SubsDev L, double zw, const double *tab, const int *ixs, int nx, const int *iys, int ny,
                            double *out) {
    const int q = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (q >= nx * ny) return;                  // whole warps: blockDim is a multiple of 32
    const int mx = L.mx, my = L.my;
    const int ixo = ixs[q % nx] - 1, iyo = iys[q / nx] - 1;
    const int ia = (zw >= 0.0) ? 0 : 1, neg = (zw >= 0.0) ? 1 : -1;
    const size_t bs = (size_t)4 * mx * my;
    double vr[3][4] = {};
    for (int jj = lane; jj < mx * my; jj += 32) {
        const int jx = jj % mx, jy = jj / mx;
        const double p[3] = {(ia == 1 ? -1.0 : 1.0) * L.px[jj], L.py[jj], L.pn[jj]};
        if (p[0] == 0.0 && p[1] == 0.0 && p[2] == 0.0) continue;
        const size_t o = (size_t)(ixo - jx + mx) + (size_t)(iyo - jy + my) * 2 * mx;
        for (int k = 0; k < 4; k++)
            for (int j = 0; j < 3; j++) {
                const double *b = tab + (size_t)(9 * k + 3 * j) * bs + o;
                vr[j][k] += b[0] * p[0] + b[bs] * p[1] + b[2 * bs] * p[2];
            }
    }
    warp_sum12(vr);
    if (lane == 0) subs_derived(L.gg[ia], L.poiss[ia], neg, vr, out + (size_t)18 * q);
}

} // namespace cgb

namespace {

// the surface load in device memory, freed in the destructor
struct DevLoad {
    cgb::SubsDev d{};
    double *buf = nullptr;
    cudaError_t init(const cgb::SubsLoad &L, cudaStream_t st) {
        const size_t n = (size_t)L.mx * L.my;
        cudaError_t e = cudaMallocAsync((void **)&buf, 3 * n * sizeof(double), st);
        if (e != cudaSuccess) return e;
        if ((e = cudaMemcpyAsync(buf, L.pn, n * sizeof(double), cudaMemcpyHostToDevice, st)) != cudaSuccess) return e;
        if ((e = cudaMemcpyAsync(buf + n, L.px, n * sizeof(double), cudaMemcpyHostToDevice, st)) != cudaSuccess) return e;
        if ((e = cudaMemcpyAsync(buf + 2 * n, L.py, n * sizeof(double), cudaMemcpyHostToDevice, st)) != cudaSuccess)
            return e;
        d.mx = L.mx; d.my = L.my; d.dx = L.dx; d.dy = L.dy; d.xc1 = L.xc1; d.yc1 = L.yc1;
        d.pn = buf; d.px = buf + n; d.py = buf + 2 * n;
        d.gg[0] = L.gg[0]; d.gg[1] = L.gg[1]; d.poiss[0] = L.poiss[0]; d.poiss[1] = L.poiss[1];
        return cudaSuccess;
    }
    void release(cudaStream_t st) { if (buf) cudaFreeAsync(buf, st); buf = nullptr; }
};

// points per CTA of the summing kernels (one warp each); threads per CTA of the table kernel
// (four per table offset; a multiple of 32, so that its shuffles see whole warps)
constexpr int kSubsWarps = 4, kSubsTableThreads = 64;

} // namespace

namespace cgb {

int subs_points(const SubsLoad &L, int npts, const double *xyz, double *out) {
    if (npts <= 0) return 0;
    cudaStream_t st = cudaStreamPerThread;
    DevLoad dl;
    cudaError_t e = dl.init(L, st);
    double *dxyz = nullptr, *dout = nullptr;
    if (e == cudaSuccess) e = cudaMallocAsync((void **)&dxyz, (size_t)3 * npts * sizeof(double), st);
    if (e == cudaSuccess) e = cudaMallocAsync((void **)&dout, (size_t)kSubsCols * npts * sizeof(double), st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(dxyz, xyz, (size_t)3 * npts * sizeof(double), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) {
        k_subs_points<<<(npts + kSubsWarps - 1) / kSubsWarps, 32 * kSubsWarps, 0, st>>>(dl.d, dxyz, npts, dout);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(out, dout, (size_t)kSubsCols * npts * sizeof(double), cudaMemcpyDeviceToHost, st);
    if (dxyz) cudaFreeAsync(dxyz, st);
    if (dout) cudaFreeAsync(dout, st);
    dl.release(st);
    const cudaError_t es = cudaStreamSynchronize(st);
    if (e == cudaSuccess) e = es;
    if (e == cudaSuccess) count_launches(1);
    return (int)e;
}

int subs_depth(const SubsLoad &L, double zw, int nx, const int *ixs, int ny, const int *iys, double *out) {
    if (nx <= 0 || ny <= 0) return 0;
    cudaStream_t st = cudaStreamPerThread;
    const int mx = L.mx, my = L.my, npts = nx * ny;
    DevLoad dl;
    cudaError_t e = dl.init(L, st);
    double *tab = nullptr, *dout = nullptr;
    int *dix = nullptr;
    const size_t tabn = (size_t)36 * 4 * mx * my;
    if (e == cudaSuccess) e = cudaMallocAsync((void **)&tab, tabn * sizeof(double), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(tab, 0, tabn * sizeof(double), st);
    if (e == cudaSuccess) e = cudaMallocAsync((void **)&dix, (size_t)(nx + ny) * sizeof(int), st);
    if (e == cudaSuccess) e = cudaMallocAsync((void **)&dout, (size_t)kSubsCols * npts * sizeof(double), st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dix, ixs, (size_t)nx * sizeof(int), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dix + nx, iys, (size_t)ny * sizeof(int), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) {
        const long long nt = 4LL * (mx + 1) * (my + 1);
        k_subs_table<<<(unsigned)((nt + kSubsTableThreads - 1) / kSubsTableThreads), kSubsTableThreads, 0, st>>>(
            dl.d, zw, tab);
        k_subs_conv<<<(npts + kSubsWarps - 1) / kSubsWarps, 32 * kSubsWarps, 0, st>>>(dl.d, zw, tab, dix, nx,
                                                                                     dix + nx, ny, dout);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(out, dout, (size_t)kSubsCols * npts * sizeof(double), cudaMemcpyDeviceToHost, st);
    if (tab) cudaFreeAsync(tab, st);
    if (dix) cudaFreeAsync(dix, st);
    if (dout) cudaFreeAsync(dout, st);
    dl.release(st);
    const cudaError_t es = cudaStreamSynchronize(st);
    if (e == cudaSuccess) e = es;
    if (e == cudaSuccess) count_launches(2);
    return (int)e;
}

} // namespace cgb
