// C-ABI of the GB300 contact library: CONTACT's cntc_* interface for module 3
// (src/contact_addon.f90, prototypes in matlab_intfc/contact_addon.h) on top of the
// device engine.  All arguments are passed by pointer as in the Fortran bind(c)
// interface; inputs are in the caller's unit convention (CNTC_if_units) and are
// converted to CONTACT's internal units (mm, N, rad).
//
// Per-problem state lives on the host: one Problem per (ire, icp) holds the settings
// staged by the setters and the results of the last cntc_calculate, read back by the
// getters.  cntc_calculate prepares a PatchDesc (Hertz solution, grid, solver flags),
// runs the engine on the GPU and copies the results back.  cntc_calculate_batch does the
// same for many problems with one pass of the engine.
#include <cuda_runtime.h>
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <deque>
#include <thread>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <functional>
#include <string>
#include <vector>
#include "../../include/contact_addon.h"
#include "engine_api.h"
#include "hertz.hpp"

using namespace cgb;

namespace {

// codes of src/caddon_flags.inc
constexpr int CNTC_if_units = 1933, CNTC_un_cntc = 1934, CNTC_un_spck = 1935, CNTC_un_si = 1936, CNTC_un_imper = 1937;
constexpr int CNTC_ic_config = 1967, CNTC_ic_pvtime = 1970, CNTC_ic_bound = 1971, CNTC_ic_tang = 1972,
              CNTC_ic_norm = 1973, CNTC_ic_force = 1974, CNTC_ic_frclaw = 1976, CNTC_ic_discns = 1977,
              CNTC_ic_inflcf = 1978, CNTC_ic_mater = 1979, CNTC_ic_exrhs = 1980, CNTC_ic_xflow = 1981,
              CNTC_ic_heat = 1982, CNTC_ic_iestim = 1983, CNTC_ic_output = 1984, CNTC_ic_flow = 1985,
              CNTC_ic_return = 1986, CNTC_ic_matfil = 1987, CNTC_ic_sens = 1988;
constexpr int CNTC_if_idebug = 2000, CNTC_if_wrtinp = 2002, CNTC_if_openmp = 2003, CNTC_if_timers = 2004,
              CNTC_if_ncase = 2005;
constexpr int CNTC_fld_h = 1, CNTC_fld_mu = 2, CNTC_fld_px = 3, CNTC_fld_py = 4, CNTC_fld_pn = 5, CNTC_fld_ux = 7,
              CNTC_fld_uy = 8, CNTC_fld_un = 9, CNTC_fld_taucrt = 11, CNTC_fld_uplsx = 12, CNTC_fld_uplsy = 13,
              CNTC_fld_sx = 15, CNTC_fld_sy = 16, CNTC_fld_temp1 = 20, CNTC_fld_temp2 = 21, CNTC_fld_wx = 22,
              CNTC_fld_wy = 23;
constexpr int CNTC_err_norm = -27, CNTC_err_tang = -28, CNTC_err_icp = -31, CNTC_err_other = -99;
constexpr int kMaxReid = 100, kMaxCpid = 9;
constexpr int kCaddonVersion = 100 * 25 + 10 * 2 + 0;     // version 25.2.0 of the interface

// one block of subsurface points (subs_addBlock, src/contact_addon.f90:3330-3515, and
// expand_xb, m_subsurf.f90:440-620): element centres selected by index (types 1-3, 5-7) or
// explicit x, y lists (type 9), at a regular (1-3) or listed (5-7, 9) set of depths z
struct SubsBlock {
    int isubs = 0;
    int ixl = 1, ixinc = 1, ixh = 99999, iyl = 1, iyinc = 1, iyh = 99999;
    std::vector<int> ixlist, iylist;      // types 3, 7: sorted unique positive indices
    std::vector<double> x, y, z;          // type 9: x, y; types 5-7, 9: z (internal units)
    int nz = 1;
    double zl = 0.0, dz = 1.0;            // types 1-3
    // filled by subs_calculate: effective point counts and the results, npoint rows of 21
    // columns (x, y, z, ux, uy, uz, sighyd, sigvm, sigtr, sigma1..3, the stress tensor by columns)
    int nx_eff = 0, ny_eff = 0;
    std::vector<double> table;
};

struct Problem {
    int ire = 0, icp = 0, ncase = 0;
    // unit scaling (cntc_select_units, src/m_global_data.f90:463-526)
    int units = CNTC_un_cntc;
    double s_len = 1, s_area = 1, s_forc = 1, s_veloc = 1, s_angle = 1, s_body = 1;
    // control digits (ic_init + cntc_activate_gd defaults)
    int pvtime = 2, bound = 0, tang = 3, norm = 0, force3 = 0, iestim = 0, gausei_eff = 0;
    int mater = 0, gencr = 2, rztang = 0, frclaw = 0, varfrc = 0, sens = 1, heat = 0, stress = 0;
    int output = 0, flow = 1, matfil = 0, ret = 1;
    // solver settings (solv_init, m_hierarch_data.f90:1722-1755)
    int maxgs = 999, maxin = 20, maxnr = 25, maxout = 1, mxsens = 30, inislp = 0;
    double eps = 1e-5, epsens = 1e-4, omegah = 0.9, omegas = 1.0, omgslp = 0.5;
    int gd_meth = 1, kdown = 3, kdowfb = 1;
    double fdecay = 0.9, betath = 0.1, d_ifc = 1.0, d_lin = 1.0, d_cns = 1.0, d_slp = 1.0, pow_s = 0.9;
    // material (mater_init)
    double poiss[2] = {0.28, 0.28}, gg[2] = {1.0, 1.0};
    // friction (fric_init): Coulomb
    double fstat = 0.3, fkin = 0.3, muscal = 0.3;
    // kinematics (kincns_init)
    double veloc = 1e3, chi = 0.0, dq = 2.0, dt = 1.0, cksi = 0, ceta = 0, cphi = 0, fn = 0, pen = 0, fxrel = 0,
           fyrel = 0;
    // potential contact (potcon_init) and Hertz data
    int ipotcn = 1, mx = 1, my = 1;
    double xl = -1, yl = -1, xc1 = 0, yc1 = 0, dx = 2, dy = 2, xh = 1, yh = 1, xcm = 0, ycm = 0;
    double hz_a1 = 0, hz_b1 = 0, hz_aa = 0, hz_bb = 0, hz_aob = 1, hz_scale = 1, hz_rho = 0, hz_cp = 0;
    // undeformed distance
    int ibase = 1;
    std::vector<double> prmudf = std::vector<double>(6, 0.0);
    // engine settings (library extensions CNTC_if_mixedprec, CNTC_if_groupctas)
    int mixed = 0;
    int group = 0;
    double eps32 = 1e-5;
    // results of the last calculation
    bool have = false;
    int r_mx = 0, r_my = 0, ierror = 0, itnorm = 0, ittang = 0, itcg = 0, itgs = 0, solver = 0;
    double r_dx = 0, r_dy = 0, r_xc1 = 0, r_yc1 = 0, r_dq = 1;
    double f_n = 0, f_x = 0, f_y = 0, m_z = 0, r_pen = 0, elen = 0, pmax = 0;
    int ncon = 0, nadh = 0, nslip = 0;
    // sensitivities of the last solve [out * 4 + in]: out Fn, Fx/(mu Fn), Fy/(mu Fn), Mz; in pen, cksi,
    // ceta, cphi (internal units)
    double sens_all[16] = {0};
    std::vector<double> fields;   // W_H .. W_SN columns, npot each
    std::vector<int> igs;
    std::vector<double> stats;           // engine statistics: convolution counts, status, phase cycles
    double tcpu = 0, twall = 0;
    // device cache of the influence coefficients and spectra (cntc_calculate, _batch, _async):
    // they depend only on the grid, dx, dy and the material, and are reused while that key
    // stays the same
    char key[256] = {0};          // geometry key of the cached influence coefficients
    bool ic_valid = false;
    void *d_ic = nullptr;
    size_t cap_ic = 0;
    int ic_dev = -1;
    // device copy of the last solution (px, py, pn, element division; prev_bytes layout): the
    // initial estimate of the next solve (IESTIM) and its previous time instance (P = 0, 1)
    // without a trip through host memory.  prev_key: grid of that solution.
    double *d_prev = nullptr;
    size_t cap_prev = 0;
    int prev_dev = -1;
    bool prev_valid = false;
    char prev_key[160] = {0};
    // subsurface stress blocks (subs_addBlock) and their results (subs_calculate)
    std::vector<SubsBlock> subs;
    std::mutex busy;
    // frees the device caches (cntc_finalize, cntc_finalizelast; not at process exit, when
    // the CUDA runtime may already be gone and the driver reclaims the memory)
    void release_device();
};

// bytes of device memory held by the problems' caches (coefficients and previous solutions),
// counted against the serving admission budget
std::atomic<long long> g_cache_bytes(0);

void Problem::release_device() {
    if (d_ic) { cudaFree(d_ic); g_cache_bytes -= (long long)cap_ic; }
    d_ic = nullptr; cap_ic = 0; ic_valid = false;
    if (d_prev) { cudaFree(d_prev); g_cache_bytes -= (long long)cap_prev; }
    d_prev = nullptr; cap_prev = 0; prev_valid = false;
}

std::mutex g_mu;
std::map<long, std::unique_ptr<Problem>> g_problems;
int g_initialized = -3;
int g_debug = 0;

long pkey(int ire, int icp) { return (long)ire * 100 + icp; }

Problem *lookup(int ire, int icp, bool create) {
    if (ire <= 0 || ire > 10000 || icp <= 0 || icp > kMaxCpid) return nullptr;
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_problems.find(pkey(ire, icp));
    if (it != g_problems.end()) return it->second.get();
    if (!create) return nullptr;
    auto p = std::make_unique<Problem>();
    p->ire = ire; p->icp = icp;
    Problem *r = p.get();
    g_problems[pkey(ire, icp)] = std::move(p);
    return r;
}

void log_msg(const char *msg) {
    if (g_debug >= 1) std::fprintf(stderr, "contact_gb300: %s\n", msg);
}

void select_units(Problem &p, int units) {
    if (units == CNTC_un_spck) { p.s_len = 1e3; p.s_area = 1e6; p.s_forc = 1; p.s_veloc = 1e3; p.s_angle = 1; p.s_body = -1; }
    else if (units == CNTC_un_si) { p.s_len = 1e3; p.s_area = 1e6; p.s_forc = 1; p.s_veloc = 1e3; p.s_angle = 1; p.s_body = 1; }
    else if (units == CNTC_un_cntc || units == CNTC_un_imper) { p.s_len = 1; p.s_area = 1; p.s_forc = 1; p.s_veloc = 1; p.s_angle = 1; p.s_body = 1; }
    else return;
    p.units = units;
}

// ------------------------------------------------------------------------------------------
// preparation of one patch: Hertz solution, potential contact, flags -> PatchDesc.
// Returns 0 or an error code (cntc ierror convention).
// ------------------------------------------------------------------------------------------
// coefficient blocks of a problem's patch (PatchDesc::ncf): 4, or 6 / 8 for non-identical
// materials (K != 0) in shifts / steady rolling
int ncf_of(const Problem &p) {
    const double ga = 2.0 / (1.0 / p.gg[0] + 1.0 / p.gg[1]);
    const double ak = (ga / 4.0) * ((1.0 - 2.0 * p.poiss[0]) / p.gg[0] - (1.0 - 2.0 * p.poiss[1]) / p.gg[1]);
    if (std::fabs(ak) < 1e-6) return 4;
    return p.tang == 3 ? 8 : 6;
}

struct Prep {
    PatchDesc d;
    bool ic_needed;
    bool upload;          // io block carries inputs (element-wise h or warm start)
};

int latency_ctas(int mx, int my, int fx, int fy);

// latency: the call solves this patch alone (a single cntc_calculate); with CNTC_if_groupctas
// = -1 a cooperative group of CTAs then takes it when that was timed faster for its size class
// (latency_ctas).  Batches, serving passes and the default (0) keep one CTA per patch.
int prepare(Problem &p, Prep &out, bool latency = false) {
    std::memset(&out.d, 0, sizeof(PatchDesc));
    PatchDesc &d = out.d;
    // combined material constants, combin_mater (m_hierarch_data.f90:1543-1553)
    const double ga = 2.0 / (1.0 / p.gg[0] + 1.0 / p.gg[1]);
    const double nu = ga * (p.poiss[0] / p.gg[0] + p.poiss[1] / p.gg[1]) / 2.0;
    const double ak = (ga / 4.0) * ((1.0 - 2.0 * p.poiss[0]) / p.gg[0] - (1.0 - 2.0 * p.poiss[1]) / p.gg[1]);
    // K != 0 couples the normal and tangential problems (|K| >= 1e-6, m_visc.f90:431-604): shifts
    // and steady rolling are solved; transient rolling with coupling is not provided here
    const bool cpl = std::fabs(ak) >= 1e-6;
    if (cpl && p.tang == 2) {
        log_msg("transient rolling (T=2) of non-identical materials (K != 0) is not supported");
        return CNTC_err_other;
    }
    if (p.mater != 0 || p.frclaw != 0 || p.rztang != 0 || p.varfrc != 0) {
        log_msg("only M=0, L=0, E=0 are supported");
        return CNTC_err_other;
    }
    if (p.heat == 3) { log_msg("temperatures (H=3) are not computed by this library"); return CNTC_err_other; }
    if (p.gencr >= 3) {
        log_msg("influence coefficients: only piecewise-constant loading (C=2) is supported");
        return CNTC_err_other;
    }
    if (!(p.bound == 0 || p.bound == 2 || p.bound == 3)) { log_msg("B digit not supported"); return CNTC_err_other; }
    // potential contact and Hertz (hzsol m_hertz.f90:29-93, potcon_hertz, potcon_fill)
    int ihertz = 0;
    double xl, yl, dx, dy;
    int mx = p.mx, my = p.my;
    p.hz_rho = p.hz_cp = 0.0;
    double fn = p.fn, pen = p.pen;
    if (p.ipotcn <= -1 && p.ipotcn >= -3) {
        hz::Result h;
        h.a1 = p.hz_a1; h.b1 = p.hz_b1; h.aa = p.hz_aa; h.bb = p.hz_bb; h.fn = fn; h.pen = pen;
        const double e_star = ga / (1.0 - nu);
        if (p.ipotcn == -2) hz::calc_aob(e_star, p.norm, p.hz_aob, h);
        else hz::calc3d(e_star, p.ipotcn, p.norm, h);
        p.hz_a1 = h.a1; p.hz_b1 = h.b1; p.hz_aa = h.aa; p.hz_bb = h.bb; p.hz_rho = h.rho; p.hz_cp = h.cp;
        if (p.ipotcn != -2) p.hz_aob = (h.aa <= 1e-20 && h.bb <= 1e-20) ? 1.0 : h.aa / h.bb;
        fn = h.fn; pen = h.pen;
        xl = -p.hz_scale * std::max(1e-9, h.aa);
        yl = -p.hz_scale * std::max(1e-9, h.bb);
        dx = (-2.0 * xl) / mx; dy = (-2.0 * yl) / my;
        ihertz = -p.ipotcn;
    } else if (p.ipotcn >= 1 && p.ipotcn <= 4) {
        xl = p.xl; yl = p.yl; dx = p.dx; dy = p.dy;
    } else {
        log_msg("potential contact specification not supported");
        return CNTC_err_other;
    }
    // check_roll_stepsize (m_sdis.f90:125-206)
    double chi = p.chi, dq = p.dq, veloc = p.veloc;
    const bool is_roll = p.tang == 2 || p.tang == 3;
    if (p.tang == 3 && p.gausei_eff != 2) {
        if (std::fabs(chi) > 0.01 && std::fabs(chi - M_PI) > 0.01) chi = 0.0;
        dq = dx;
    }
    if (!is_roll) { chi = 0.0; dq = 1.0; veloc = 1.0; }
    if (is_roll && std::fabs(chi) > 0.01) { log_msg("rolling direction chi != 0 is not supported"); return CNTC_err_other; }
    p.dt = dq / std::max(1e-10, veloc);
    // a single column in rolling direction is solved for the normal problem alone (FFT length 2
    // in x, as for single rows in y); with a tangential problem (ConvexGS in the reference) the
    // one-column tangential operators are not verified, so it is refused
    if ((mx < 2 && p.tang != 0) || mx < 1 || my < 1) {
        log_msg("grids with mx < 2 are supported for the normal problem only");
        return CNTC_err_other;
    }
    const int fx = cgb::opt_fft_size(mx), fy = cgb::opt_fft_size(my);
    // one CTA per patch while its FFT lines fit the per-warp buffers, a cooperative group of
    // CTAs for larger grids (or when CNTC_if_groupctas asks for one)
    const int nblk = (latency && p.group == -1) ? latency_ctas(mx, my, fx, fy)
                                                : cgb::group_size(mx, my, fx, fy, std::max(0, p.group));
    if (nblk < 1) { log_msg("patch too large for the device (shared memory of one FFT line)"); return CNTC_err_other; }
    d.nblk = nblk;
    d.mx = mx; d.my = my; d.npot = mx * my; d.fx = fx; d.fy = fy;
    d.dx = dx; d.dy = dy; d.dxdy = dx * dy; d.xc1 = xl + 0.5 * dx; d.yc1 = yl + 0.5 * dy;
    d.tang = p.tang; d.norm = p.norm; d.bound = p.bound; d.iestim = p.iestim; d.force3 = p.force3;
    d.gausei = p.gausei_eff;
    d.maxgs = p.maxgs; d.maxin = p.maxin;
    int maxout = p.maxout;
    if (maxout >= 2 && std::fabs(ak) < 1e-4) maxout = 1;
    d.maxout = maxout;
    d.eps = p.eps;
    d.omegah = p.omegah; d.omegas = p.omegas;
    d.gd_meth = p.gd_meth; d.kdown = p.kdown; d.kdowfb = p.kdowfb;
    d.fdecay = p.fdecay; d.betath = p.betath; d.d_ifc = p.d_ifc; d.d_lin = p.d_lin; d.d_cns = p.d_cns;
    d.d_slp = p.d_slp; d.pow_s = p.pow_s;
    d.ga = ga; d.nu = nu; d.ak = cpl ? ak : 0.0; d.fstat = p.fstat;
    d.ncf = ncf_of(p);
    d.chi = chi; d.dq = dq; d.cksi = p.cksi; d.ceta = p.ceta; d.cphi = p.cphi;
    d.fntrue = fn; d.pen = pen;
    d.ihertz = ihertz; d.aa = p.hz_aa; d.bb = p.hz_bb;
    if (ihertz >= 1) {
        d.ibase = 1;
        for (int k = 0; k < 6; k++) d.prm[k] = 0.0;
        d.prm[0] = p.hz_a1; d.prm[2] = p.hz_b1;
    } else {
        d.ibase = p.ibase;
        if (p.ibase == 1) for (int k = 0; k < 6; k++) d.prm[k] = p.prmudf[k];
        else if (p.ibase != 9) { log_msg("undeformed distance type not supported"); return CNTC_err_other; }
        if (p.ibase == 9 && (int)p.prmudf.size() < d.npot) return CNTC_err_other;
    }
    d.precision = p.mixed;
    d.eps32 = std::max(p.eps, p.eps32);
    d.maxnr = p.maxnr;
    d.pvtime = p.pvtime;
    d.fxrel = p.fxrel; d.fyrel = p.fyrel;
    for (int k = 0; k < 16; k++) d.sens0[k] = p.sens_all[k];
    d.sens = p.sens; d.mxsens = p.mxsens; d.epsens = p.epsens;
    // geometry key for reuse of influence coefficients and spectra
    char key[256];
    std::snprintf(key, sizeof(key), "%d %d %.17g %.17g %.17g %.17g %.17g %d %.17g", mx, my, dx, dy, ga, nu, d.ak,
                  d.ncf, d.ncf == 8 ? dq : 0.0);
    if (std::strcmp(key, p.key) != 0) p.ic_valid = false;    // the cache holds another geometry
    out.ic_needed = !p.ic_valid;
    std::strcpy(p.key, key);
    // continuation from the previous time instance (P = 0) of shifts and transient rolling
    // reads the previous tractions element by element: the grid must be the one of that solve
    // (the reference also moves them with a potential contact that moves by whole elements;
    // that form is not provided here)
    if (p.pvtime == 0 && (p.tang == 1 || p.tang == 2) && p.have &&
        !(p.r_mx == mx && p.r_my == my && p.r_dx == dx && p.r_dy == dy && p.r_xc1 == d.xc1 && p.r_yc1 == d.yc1)) {
        log_msg("continuation from the previous time instance on a moved or changed grid is not supported");
        return CNTC_err_other;
    }
    // warm start needs a previous solution on the same grid
    out.upload = (d.ibase == 9);
    if (p.iestim != 0) {
        if (!(p.have && p.r_mx == mx && p.r_my == my)) d.iestim = 0;
        else out.upload = true;
    }
    p.r_mx = mx; p.r_my = my; p.r_dx = dx; p.r_dy = dy; p.r_xc1 = d.xc1; p.r_yc1 = d.yc1; p.r_dq = dq;
    return 0;
}

// fill the io staging block of one patch with its inputs
// warm: stage the initial estimate from the host copy of the last result (false when the
// solve reads the problem's device copy instead)
void stage_inputs(Problem &p, const PatchDesc &d, double *io, bool warm = true) {
    const int n = d.npot;
    if (d.ibase == 9) for (int i = 0; i < n; i++) io[(size_t)W_H * n + i] = p.prmudf[i] * 1.0;
    if (warm && d.iestim != 0 && p.have) {
        int *igs = (int *)(io + (size_t)kIoCols * n + O_NSCAL);
        double *px = io + (size_t)W_PX * n, *py = io + (size_t)W_PY * n, *pn = io + (size_t)W_PN * n;
        for (int i = 0; i < n; i++) {
            igs[i] = p.igs[i];
            px[i] = p.fields[(size_t)W_PX * n + i];
            py[i] = p.fields[(size_t)W_PY * n + i];
            pn[i] = p.fields[(size_t)W_PN * n + i];
            // I = 1: regularise tractions (init_curr_data, m_sdis.f90:716-729)
            if (p.iestim == 1) {
                if (igs[i] <= 0) { pn[i] = px[i] = py[i] = 0.0; }
                else if (igs[i] == 2) {
                    const double pabs = std::max(1e-10, std::sqrt(px[i] * px[i] + py[i] * py[i]));
                    px[i] = p.fstat * pn[i] * px[i] / pabs;
                    py[i] = p.fstat * pn[i] * py[i] / pabs;
                }
            }
            if (p.iestim == 2) { if (igs[i] >= 1) igs[i] = 1; px[i] = py[i] = 0.0; }
        }
    }
}

// copy the results of one patch out of its io block
void collect(Problem &p, const PatchDesc &d, const double *io) {
    const int n = d.npot;
    const double *o = io + (size_t)kIoCols * n;
    p.fields.assign(io, io + (size_t)kIoCols * n);
    const int *igs = (const int *)(o + O_NSCAL);
    p.igs.assign(igs, igs + n);
    p.f_n = o[O_FN]; p.f_x = o[O_FX]; p.f_y = o[O_FY]; p.m_z = o[O_MZ];
    p.r_pen = o[O_PEN]; p.pmax = o[O_PMAX];
    // the normal problem is skipped for B = 2..4 and its elastic energy is reported as zero
    // (m_soutpt.f90:453-458)
    p.elen = (d.bound >= 2 && d.bound <= 4) ? 0.0 : o[O_ELEN];
    p.ierror = (int)o[O_IERR]; p.itnorm = (int)o[O_ITNORM]; p.ittang = (int)o[O_ITTANG];
    p.itcg = (int)o[O_ITCG]; p.itgs = (int)o[O_ITGS]; p.solver = (int)o[O_SOLVER];
    p.ncon = (int)o[O_NCON]; p.nadh = (int)o[O_NADH]; p.nslip = (int)o[O_NSLIP];
    p.stats.assign(o + O_NCONV32, o + O_TEND + 1);
    p.stats.push_back((double)d.nblk);
    // total forces prescribed: the creepages found by the Newton-Raphson and its sensitivities
    // (the reference keeps them in the problem's kinematics and output, m_solvpt.f90:51-378)
    if (d.tang != 0 && d.force3 >= 1) {
        p.cksi = o[O_CKSI];
        if (d.force3 >= 2) p.ceta = o[O_CETA];
    }
    for (int k = 0; k < 16; k++) p.sens_all[k] = o[O_SENS + k];
    p.have = true;
    // kinematic outputs follow the reference: fn from the solution when N = 0
    if (p.norm == 0) p.fn = p.f_n;
    p.pen = p.r_pen;
}

// ------------------------------------------------------------------------------------------
// batched execution of prepared problems (one pass of the engine)
// ------------------------------------------------------------------------------------------
struct Batch {
    std::vector<Problem *> probs;
    std::vector<Prep> preps;
    std::vector<int> status;
};

struct Arena {
    char *d_io = nullptr, *d_work = nullptr;
    size_t cap_io = 0, cap_work = 0;
    PatchDesc *d_desc = nullptr;
    size_t cap_desc = 0;
    int *d_list = nullptr;
    size_t cap_list = 0;
    double *h_io = nullptr;      // pinned staging
    size_t cap_hio = 0;
    // per-patch completion flags in host-mapped memory (h_flags, seen by the device as
    // d_flags) and the stream that copies finished patches back while the pass runs
    int *h_flags = nullptr, *d_flags = nullptr;
    size_t cap_flags = 0;
    cudaStream_t copy_st = nullptr;
    // pinned host buffers replaced by larger ones: freeing pinned memory synchronises the whole
    // device, which would stall every other pass in flight, so they are kept until the thread
    // that owns the arena exits
    std::vector<void *> retired_host;
    // at thread exit: the arena's passes have all completed (each call waits for its own), so
    // its buffers and stream are released here, not leaked with the thread
    ~Arena() {
        for (void *q : retired_host) cudaFreeHost(q);
        if (h_io) cudaFreeHost(h_io);
        if (h_flags) cudaFreeHost(h_flags);
        for (void *q : {(void *)d_io, (void *)d_work, (void *)d_desc, (void *)d_list})
            if (q) cudaFree(q);
        if (copy_st) cudaStreamDestroy(copy_st);
    }
};

// Device buffers come from the stream-ordered allocator on the caller's stream: a replaced
// buffer is released after the work queued before it on that stream, without the device-wide
// synchronisation of cudaFree (other threads' passes keep running).
cudaError_t grow(void **ptr, size_t &cap, size_t need, bool pinned, cudaStream_t st, std::vector<void *> &retired) {
    if (need <= cap) return cudaSuccess;
    if (*ptr) {
        if (pinned) retired.push_back(*ptr);
        else cudaFreeAsync(*ptr, st);
        *ptr = nullptr; cap = 0;
    }
    size_t c = need + need / 4 + 4096;
    cudaError_t e = pinned ? cudaMallocHost(ptr, c) : cudaMallocAsync(ptr, c, st);
    if (e == cudaSuccess) cap = c;
    return e;
}

thread_local Arena t_arena;
// bytes moved by the last host<->device batch copy of this thread
thread_local long long t_h2d_bytes = 0, t_d2h_bytes = 0;

// runs the engine for all prepared entries with status 0; results go to the problems.
// on_done (serving): called with the batch index of each patch as soon as its results are in
// its problem, while the rest of the pass still runs; patches the pass leaves without a
// completion flag (early returns) are collected when the pass has ended
int run_batch(Batch &b, Arena &A, bool reuse_ic_allowed, const std::function<void(int)> *on_done = nullptr) {
    const auto tb0 = std::chrono::steady_clock::now();
    std::vector<int> live;
    for (size_t i = 0; i < b.probs.size(); i++) if (b.status[i] == 0) live.push_back((int)i);
    const int n = (int)live.size();
    if (n == 0) return 0;
    std::vector<size_t> off_io(n), off_work(n);
    size_t tot_io = 0, tot_work = 0;
    bool any_upload = false;
    for (int k = 0; k < n; k++) {
        const PatchDesc &d = b.preps[live[k]].d;
        PatchSizes s = patch_sizes(d.mx, d.my, d.fx, d.fy, d.nblk, d.ncf);
        off_io[k] = tot_io; tot_io += s.io;
        off_work[k] = tot_work; tot_work += s.work;
        any_upload |= b.preps[live[k]].upload;
    }
    cudaError_t e;
    const cudaStream_t gst = cudaStreamPerThread;
    auto &rt = A.retired_host;
    if ((e = grow((void **)&A.d_io, A.cap_io, tot_io, false, gst, rt)) != cudaSuccess) return (int)e;
    if ((e = grow((void **)&A.d_work, A.cap_work, tot_work, false, gst, rt)) != cudaSuccess) return (int)e;
    if ((e = grow((void **)&A.d_desc, A.cap_desc, n * sizeof(PatchDesc), false, gst, rt)) != cudaSuccess) return (int)e;
    if ((e = grow((void **)&A.d_list, A.cap_list, 3 * n * sizeof(int) + 64, false, gst, rt)) != cudaSuccess)
        return (int)e;
    if ((e = grow((void **)&A.h_io, A.cap_hio, tot_io, true, gst, rt)) != cudaSuccess) return (int)e;
    std::vector<PatchDesc> hd(n);
    std::vector<unsigned char> need_ic(n, 1);
    std::vector<int> ic_fill;     // patches whose coefficient cache this pass fills
    std::vector<unsigned char> dev_prev(n, 0);   // patches that start from their device copy
    int dev = 0;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return (int)e;
    for (int k = 0; k < n; k++) {
        hd[k] = b.preps[live[k]].d;
        carve_patch(hd[k], A.d_io + off_io[k], A.d_work + off_work[k]);
        if (reuse_ic_allowed) {
            // coefficients and spectra live in the problem's own device buffer: reused when
            // the geometry is unchanged, computed into it otherwise (without a buffer, when
            // the allocation fails, they are computed in the pass's work area as before)
            Problem &p = *b.probs[live[k]];
            const PatchSizes ps = patch_sizes(hd[k].mx, hd[k].my, hd[k].fx, hd[k].fy, hd[k].nblk, hd[k].ncf);
            const size_t icb = ps.cf + ps.spec64 + ps.spec32;
            const bool hit = p.ic_valid && !b.preps[live[k]].ic_needed && p.d_ic && p.ic_dev == dev && p.cap_ic >= icb;
            if (!hit) {
                p.ic_valid = false;
                if (p.d_ic && (p.cap_ic < icb || p.ic_dev != dev)) {
                    cudaFree(p.d_ic); g_cache_bytes -= (long long)p.cap_ic; p.d_ic = nullptr; p.cap_ic = 0;
                }
                if (!p.d_ic) {
                    if (cudaMalloc(&p.d_ic, icb) == cudaSuccess) { p.cap_ic = icb; p.ic_dev = dev; g_cache_bytes += (long long)icb; }
                    else { cudaGetLastError(); p.d_ic = nullptr; }
                }
                if (p.d_ic) ic_fill.push_back(k);
            } else {
                need_ic[k] = 0;
            }
            if (p.d_ic) {
                char *c = (char *)p.d_ic;
                hd[k].cf = (const double *)c;
                hd[k].spec64 = (const double *)(c + ps.cf);
                hd[k].spec32 = (const float *)(c + ps.cf + ps.spec64);
            }
            // the previous solution in device memory: read when the grid is unchanged and the
            // solve asks for it (initial estimate or previous time instance), then overwritten
            // by this solve's own solution
            const size_t pb = prev_bytes(hd[k].npot);
            char pkey[160];
            std::snprintf(pkey, sizeof(pkey), "%d %d %.17g %.17g %.17g %.17g", hd[k].mx, hd[k].my, hd[k].dx, hd[k].dy,
                          hd[k].xc1, hd[k].yc1);
            const bool want = hd[k].iestim != 0 || (hd[k].pvtime <= 1 && (hd[k].tang == 1 || hd[k].tang == 2));
            const bool prev_ok = p.prev_valid && p.d_prev && p.prev_dev == dev && std::strcmp(pkey, p.prev_key) == 0;
            if (p.d_prev && (p.cap_prev < pb || p.prev_dev != dev)) {
                cudaFree(p.d_prev); g_cache_bytes -= (long long)p.cap_prev;
                p.d_prev = nullptr; p.cap_prev = 0; p.prev_valid = false;
            }
            if (!p.d_prev) {
                if (cudaMalloc((void **)&p.d_prev, pb) == cudaSuccess) {
                    p.cap_prev = pb; p.prev_dev = dev; g_cache_bytes += (long long)pb;
                } else { cudaGetLastError(); p.d_prev = nullptr; }
            }
            if (want && prev_ok) {
                hd[k].prev = p.d_prev;
                dev_prev[k] = 1;
            }
            hd[k].save = p.d_prev;
            if (p.d_prev) { std::strcpy(p.prev_key, pkey); p.prev_valid = false; }
        }
        if (b.preps[live[k]].upload)
            stage_inputs(*b.probs[live[k]], hd[k], (double *)((char *)A.h_io + off_io[k]), !dev_prev[k]);
    }
    if (on_done) {
        if (A.cap_flags < (size_t)n) {
            if (A.h_flags) { A.retired_host.push_back(A.h_flags); A.h_flags = A.d_flags = nullptr; A.cap_flags = 0; }
            const size_t c = (size_t)n + n / 4 + 64;
            if ((e = cudaHostAlloc((void **)&A.h_flags, c * sizeof(int), cudaHostAllocMapped)) != cudaSuccess) return (int)e;
            if ((e = cudaHostGetDevicePointer((void **)&A.d_flags, A.h_flags, 0)) != cudaSuccess) return (int)e;
            A.cap_flags = c;
        }
        if (!A.copy_st && (e = cudaStreamCreateWithFlags(&A.copy_st, cudaStreamNonBlocking)) != cudaSuccess) return (int)e;
        for (int k = 0; k < n; k++) { ((volatile int *)A.h_flags)[k] = 0; hd[k].done = A.d_flags + k; }
    }
    cudaStream_t st = cudaStreamPerThread;
    const auto tb1 = std::chrono::steady_clock::now();
    t_h2d_bytes = (long long)(n * sizeof(PatchDesc));
    if (any_upload) {
        if ((e = cudaMemcpyAsync(A.d_io, A.h_io, tot_io, cudaMemcpyHostToDevice, st)) != cudaSuccess) return (int)e;
        t_h2d_bytes += (long long)tot_io;
    }
    if ((e = cudaMemcpyAsync(A.d_desc, hd.data(), n * sizeof(PatchDesc), cudaMemcpyHostToDevice, st)) != cudaSuccess)
        return (int)e;
    int rc = engine_run(hd.data(), A.d_desc, n, need_ic.data(), A.d_list, st);
    if (rc != 0) return rc;
    if (on_done) {
        std::vector<char> fin(n, 0);
        std::vector<char> icf(n, 0);
        for (int k : ic_fill) icf[k] = 1;
        t_d2h_bytes = 0;
        auto finish = [&](int k) -> cudaError_t {
            const size_t bytes = patch_sizes(hd[k].mx, hd[k].my, hd[k].fx, hd[k].fy, hd[k].nblk, hd[k].ncf).io;
            cudaError_t ce = cudaMemcpyAsync((char *)A.h_io + off_io[k], A.d_io + off_io[k], bytes,
                                             cudaMemcpyDeviceToHost, A.copy_st);
            if (ce == cudaSuccess) ce = cudaStreamSynchronize(A.copy_st);
            if (ce != cudaSuccess) return ce;
            t_d2h_bytes += (long long)bytes;
            Problem &p = *b.probs[live[k]];
            if (icf[k]) p.ic_valid = true;
            if (hd[k].save) p.prev_valid = true;
            collect(p, hd[k], (const double *)((const char *)A.h_io + off_io[k]));
            fin[k] = 1;
            (*on_done)(live[k]);
            return cudaSuccess;
        };
        int left = n;
        for (;;) {
            bool any = false;
            for (int k = 0; k < n; k++) {
                if (fin[k] || ((volatile int *)A.h_flags)[k] == 0) continue;
                if ((e = finish(k)) != cudaSuccess) return (int)e;
                left--;
                any = true;
            }
            if (left == 0) break;
            if (!any) {
                const cudaError_t q = cudaStreamQuery(st);
                if (q == cudaSuccess) break;
                if (q != cudaErrorNotReady) return (int)q;
                std::this_thread::sleep_for(std::chrono::microseconds(200));
            }
        }
        if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return (int)e;
        for (int k = 0; k < n; k++)
            if (!fin[k] && (e = finish(k)) != cudaSuccess) return (int)e;
        return 0;
    }
    if ((e = cudaMemcpyAsync(A.h_io, A.d_io, tot_io, cudaMemcpyDeviceToHost, st)) != cudaSuccess) return (int)e;
    t_d2h_bytes = (long long)tot_io;
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return (int)e;
    const auto tb2 = std::chrono::steady_clock::now();
    for (int k : ic_fill) b.probs[live[k]]->ic_valid = true;
    for (int k = 0; k < n; k++) if (hd[k].save) b.probs[live[k]]->prev_valid = true;
    for (int k = 0; k < n; k++) collect(*b.probs[live[k]], hd[k], (const double *)((const char *)A.h_io + off_io[k]));
    if (g_debug >= 2) {
        const auto tb3 = std::chrono::steady_clock::now();
        std::fprintf(stderr, "contact_gb300: batch of %d: staging %.3f s, device %.3f s, collect %.3f s\n", n,
                     std::chrono::duration<double>(tb1 - tb0).count(), std::chrono::duration<double>(tb2 - tb1).count(),
                     std::chrono::duration<double>(tb3 - tb2).count());
    }
    return 0;
}

// on_done (serving): called with (batch index, ierror) for each entry as soon as it is
// finished, after its problem has been released; entries refused before the pass are finished
// before it starts
int calculate_many(int n, const int *ire, const int *icp, int *ierror,
                   const std::function<void(int, int)> *on_done = nullptr) {
    Batch b;
    b.probs.resize(n); b.preps.resize(n); b.status.assign(n, 0);
    auto t0 = std::chrono::steady_clock::now();
    std::vector<std::unique_lock<std::mutex>> locks(n);
    std::vector<char> fin(n, 0);
    for (int i = 0; i < n; i++) {
        Problem *p = lookup(ire[i], icp[i], true);
        b.probs[i] = p;
        if (!p) { b.status[i] = CNTC_err_icp; continue; }
        std::unique_lock<std::mutex> lk(p->busy, std::try_to_lock);
        if (!lk.owns_lock()) { b.status[i] = CNTC_err_other; continue; }   // same problem in use
        locks[i] = std::move(lk);
        p->ncase++;
        b.status[i] = prepare(*p, b.preps[i], n == 1 && !on_done);
        if (b.status[i] != 0) p->have = false;
    }
    if (g_debug >= 2)
        std::fprintf(stderr, "contact_gb300: batch prepare %.3f s\n",
                     std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count());
    // an entry's result: its problem's wall time (the pass's share, or the time until the entry
    // finished in serving), then the problem is released
    auto finish = [&](int i, int e, double dt) {
        ierror[i] = e;
        if (b.probs[i] && b.status[i] == 0) { b.probs[i]->twall += dt; b.probs[i]->tcpu += dt; }
        if (locks[i].owns_lock()) locks[i].unlock();
        fin[i] = 1;
        if (on_done) (*on_done)(i, e);
    };
    if (on_done)
        for (int i = 0; i < n; i++)
            if (b.status[i] != 0) finish(i, b.status[i], 0.0);
    std::function<void(int)> cb = [&](int i) {
        finish(i, b.probs[i]->ierror,
               std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count());
    };
    int rc = run_batch(b, t_arena, true, on_done ? &cb : nullptr);
    auto t1 = std::chrono::steady_clock::now();
    const double dt = std::chrono::duration<double>(t1 - t0).count();
    for (int i = 0; i < n; i++) {
        if (fin[i]) continue;
        if (!b.probs[i] || b.status[i] != 0) { finish(i, b.status[i], 0.0); continue; }
        finish(i, (rc != 0) ? CNTC_err_other : b.probs[i]->ierror, dt / n);
    }
    if (rc != 0 && g_debug >= 1) std::fprintf(stderr, "contact_gb300: engine error %d (%s)\n", rc, cudaGetErrorString((cudaError_t)rc));
    return rc;
}

// ------------------------------------------------------------------------------------------
// launch shape of a single-patch call, tuned per size class (CNTC_if_groupctas = -1).  A patch
// solved alone by one CTA uses one SM of the device; a cooperative group of CTAs (one per 256
// elements) solves it sooner once the grid is large enough for the group barriers to pay.  The
// group's reductions sum in another order, so its results agree with the one-CTA form to
// rounding, not bit for bit; the default therefore keeps one CTA.  For each size class
// (element count in a factor-of-two band, from kLatencyMinElements to kMaxGroupGsElements, the
// largest group that still runs SteadyGS) the first single-patch call on a device times a
// synthetic normal problem of that class (Hertzian, square grid, the middle of the band) in both
// shapes and keeps the faster one.  Batches and serving passes keep one CTA per patch, which
// is the throughput form.
// ------------------------------------------------------------------------------------------
constexpr int kLatencyMinElements = 4096;
constexpr int kElementsPerCta = 256;                 // group_size: one element per thread of a CTA

struct ShapeTuner {
    std::mutex mu;
    std::map<std::pair<int, int>, int> group;      // (device, size class) -> 1: group, 0: one CTA
};
ShapeTuner &shape_tuner() {
    static ShapeTuner t;
    return t;
}

// seconds of one warm pass of the synthetic problem (side x side) with group request req
double time_shape(int side, int req) {
    Problem q;
    q.tang = 0; q.norm = 1; q.fn = 1.0; q.eps = 1e-6;
    q.ipotcn = -3; q.mx = side; q.my = side; q.hz_aa = 1.0; q.hz_bb = 1.0; q.hz_scale = 1.1;
    q.group = req;
    double best = 1e30;
    for (int rep = 0; rep < 3; rep++) {
        Batch b;
        b.probs = {&q}; b.preps.resize(1); b.status = {0};
        if (prepare(q, b.preps[0]) != 0) return 1e30;
        const auto t0 = std::chrono::steady_clock::now();
        const int rc = run_batch(b, t_arena, false);
        const double t = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        if (rc != 0) { cudaGetLastError(); return 1e30; }
        if (rep > 0) best = std::min(best, t);      // the first pass includes first-use costs
    }
    return best;
}

int latency_ctas(int mx, int my, int fx, int fy) {
    const int n = mx * my;
    const int automatic = cgb::group_size(mx, my, fx, fy, 0);
    if (n < kLatencyMinElements || n > kMaxGroupGsElements || automatic != 1) return automatic;
    int cls = 0;
    while ((2 << cls) <= n) cls++;                   // 2^cls <= n < 2^(cls + 1)
    int dev = 0;
    cudaGetDevice(&dev);
    ShapeTuner &t = shape_tuner();
    std::lock_guard<std::mutex> lk(t.mu);
    auto it = t.group.find({dev, cls});
    if (it == t.group.end()) {
        const int side = (int)std::lround(std::sqrt(1.5 * (double)(1 << cls)));
        const int g = std::max(2, (side * side + kElementsPerCta - 1) / kElementsPerCta);
        const double t1 = time_shape(side, 1), tg = time_shape(side, g);
        if (g_debug >= 1)
            std::fprintf(stderr, "contact_gb300: single-patch calls of %d..%d elements: one CTA %.4f s, "
                                 "a group of %d CTAs %.4f s\n", 1 << cls, (2 << cls) - 1, t1, g, tg);
        it = t.group.emplace(std::make_pair(dev, cls), tg < t1 ? 1 : 0).first;
    }
    if (!it->second) return 1;
    const int g = cgb::group_size(mx, my, fx, fy, std::max(2, (n + kElementsPerCta - 1) / kElementsPerCta));
    return g >= 2 ? g : 1;
}

// the sizes chosen so far, for the diagnostics of cntc_gb300_latencyshapes
int latency_shapes(int *cls, int *grp, int cap) {
    ShapeTuner &t = shape_tuner();
    std::lock_guard<std::mutex> lk(t.mu);
    int k = 0;
    for (const auto &e : t.group) {
        if (k >= cap) break;
        cls[k] = e.first.second; grp[k] = e.second; k++;
    }
    return k;
}

// ------------------------------------------------------------------------------------------
// resident batch: a set of prepared problems staged in device memory once and solved again
// and again on the same inputs (throughput with inputs already in HBM).  Each solve runs the
// whole engine, influence coefficients included.
//
// Consecutive passes overlap (continuous batching across passes): the batch is staged in
// `depth` buffer sets, each with its own caller stream and side-stream set, and pass r runs
// in set r mod depth.  The SMs that the last patches of pass r leave idle take the CTAs of
// passes r+1 .. r+depth-1; pass r+depth waits (stream order) until pass r has finished with
// its buffers.  depth 1 is the plain sequence of passes.
// ------------------------------------------------------------------------------------------
constexpr int kMaxResidentSets = 4;

struct ResSet {
    char *d_io = nullptr, *d_work = nullptr;
    PatchDesc *d_desc = nullptr;
    int *d_list = nullptr;
    std::vector<PatchDesc> hd;
    cudaStream_t st = nullptr;
    EngineTimer tm;
    bool have_events = false;
    EnginePlan plan;
    cudaGraphExec_t exec = nullptr;    // the pass captured once and replayed (null: direct launches)
};

struct Resident {
    Batch b;
    std::vector<int> live;
    std::vector<unsigned char> need_ic;
    std::vector<size_t> off_io;
    size_t tot_io = 0;
    double *h_io = nullptr;       // pinned staging
    ResSet set[kMaxResidentSets];
    int depth = 1;
    int last = 0;                 // set of the last pass
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    ~Resident() {
        for (ResSet &r : set) {
            if (r.exec) cudaGraphExecDestroy(r.exec);
            if (r.have_events) for (auto &e : r.tm.ev) cudaEventDestroy(e);
            if (r.d_io) cudaFree(r.d_io);
            if (r.d_work) cudaFree(r.d_work);
            if (r.d_desc) cudaFree(r.d_desc);
            if (r.d_list) cudaFree(r.d_list);
            if (r.st) cudaStreamDestroy(r.st);
        }
        if (ev0) cudaEventDestroy(ev0);
        if (ev1) cudaEventDestroy(ev1);
        if (h_io) cudaFreeHost(h_io);
    }
};
std::mutex g_res_mu;
std::unique_ptr<Resident> g_res;
int g_res_depth = 1;

int resident_setup(int n, const int *ire, const int *icp, int *ierror) {
    g_res.reset();
    auto R = std::make_unique<Resident>();
    R->depth = std::max(1, std::min(g_res_depth, kMaxResidentSets));
    Batch &b = R->b;
    b.probs.resize(n); b.preps.resize(n); b.status.assign(n, 0);
    for (int i = 0; i < n; i++) {
        Problem *p = lookup(ire[i], icp[i], true);
        b.probs[i] = p;
        if (!p) { b.status[i] = CNTC_err_icp; continue; }
        b.status[i] = prepare(*p, b.preps[i]);
    }
    for (int i = 0; i < n; i++) { ierror[i] = b.status[i]; if (b.status[i] == 0) R->live.push_back(i); }
    const int m = (int)R->live.size();
    std::vector<size_t> off_work(m);
    R->off_io.resize(m);
    size_t tot_work = 0;
    for (int k = 0; k < m; k++) {
        const PatchDesc &d = b.preps[R->live[k]].d;
        PatchSizes s = patch_sizes(d.mx, d.my, d.fx, d.fy, d.nblk, d.ncf);
        R->off_io[k] = R->tot_io; R->tot_io += s.io;
        off_work[k] = tot_work; tot_work += s.work;
    }
    cudaError_t e;
    if ((e = cudaMallocHost((void **)&R->h_io, std::max<size_t>(R->tot_io, 256))) != cudaSuccess) return (int)e;
    R->need_ic.assign(m, 1);
    std::vector<PatchDesc> hd0(m);
    for (int k = 0; k < m; k++) {
        hd0[k] = b.preps[R->live[k]].d;
        stage_inputs(*b.probs[R->live[k]], hd0[k], (double *)((char *)R->h_io + R->off_io[k]));
    }
    for (int si = 0; si < R->depth; si++) {
        ResSet &S = R->set[si];
        if ((e = cudaMalloc((void **)&S.d_io, std::max<size_t>(R->tot_io, 256))) != cudaSuccess) return (int)e;
        if ((e = cudaMalloc((void **)&S.d_work, std::max<size_t>(tot_work, 256))) != cudaSuccess) return (int)e;
        if ((e = cudaMalloc((void **)&S.d_desc, std::max<size_t>(m * sizeof(PatchDesc), 256))) != cudaSuccess)
            return (int)e;
        if ((e = cudaMalloc((void **)&S.d_list, 3 * m * sizeof(int) + 64)) != cudaSuccess) return (int)e;
        if ((e = cudaStreamCreateWithFlags(&S.st, cudaStreamNonBlocking)) != cudaSuccess) return (int)e;
        S.hd = hd0;
        for (int k = 0; k < m; k++) carve_patch(S.hd[k], S.d_io + R->off_io[k], S.d_work + off_work[k]);
        if ((e = cudaMemcpyAsync(S.d_io, R->h_io, R->tot_io, cudaMemcpyHostToDevice, S.st)) != cudaSuccess)
            return (int)e;
        if ((e = cudaMemcpyAsync(S.d_desc, S.hd.data(), m * sizeof(PatchDesc), cudaMemcpyHostToDevice, S.st)) !=
            cudaSuccess)
            return (int)e;
        if ((e = cudaStreamSynchronize(S.st)) != cudaSuccess) return (int)e;
        for (auto &ev : S.tm.ev) if ((e = cudaEventCreate(&ev)) != cudaSuccess) return (int)e;
        S.have_events = true;
        // launch plan and lists once; the pass (influence coefficients, spectra, the persistent
        // solve) captured into a CUDA graph that each pass replays.  Patch groups (cooperative
        // launches) keep direct launches.
        int rc = engine_plan(S.hd.data(), m, R->need_ic.data(), S.plan);
        if (rc != 0) return rc;
        if ((e = cudaMemcpyAsync(S.d_list, S.plan.all.data(), S.plan.all.size() * sizeof(int),
                                 cudaMemcpyHostToDevice, S.st)) != cudaSuccess)
            return (int)e;
        if ((e = cudaStreamSynchronize(S.st)) != cudaSuccess) return (int)e;
        if (S.plan.groups.empty()) {
            cudaGraph_t g = nullptr;
            if (cudaStreamBeginCapture(S.st, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
                rc = engine_launch(S.plan, S.d_desc, S.d_list, S.st, nullptr);
                const cudaError_t ec = cudaStreamEndCapture(S.st, &g);
                if (rc == 0 && ec == cudaSuccess && g && cudaGraphInstantiate(&S.exec, g, 0) != cudaSuccess)
                    S.exec = nullptr;
                if (g) cudaGraphDestroy(g);
            }
            cudaGetLastError();
        }
    }
    if ((e = cudaEventCreate(&R->ev0)) != cudaSuccess) return (int)e;
    if ((e = cudaEventCreate(&R->ev1)) != cudaSuccess) return (int)e;
    g_res = std::move(R);
    return 0;
}

// nrep solves of the resident batch, overlapped over the buffer sets.  Per solve r:
// times[4r] = device time of the whole sequence / nrep (CUDA events on the first set's stream,
// around all passes), times[4r+1] = span of pass r's patch-solve launches, times[4r+2] = span of
// its influence-coefficient and spectrum kernels (ms, events on the pass's stream),
// times[4r+3] = its number of launches
int resident_solve(int nrep, double *times) {
    Resident *R = g_res.get();
    if (!R || R->live.empty()) return -1;
    const int m = (int)R->live.size(), D = R->depth;
    cudaError_t e;
    cudaStream_t s0 = R->set[0].st;
    if ((e = cudaEventRecord(R->ev0, s0)) != cudaSuccess) return (int)e;
    for (int si = 1; si < D; si++)
        if ((e = cudaStreamWaitEvent(R->set[si].st, R->ev0, 0)) != cudaSuccess) return (int)e;
    std::vector<std::vector<double>> spans(nrep, std::vector<double>(3, 0.0));
    auto read_spans = [&](int r, ResSet &S) {
        const EngineTimer &tm = S.tm;
        float ms = 0.f;
        for (int k = 0; k < tm.nlaunch; k++) {
            cudaEventElapsedTime(&ms, tm.ev[2 * k], tm.ev[2 * k + 1]);
            spans[r][tm.kind[k] == 2 ? 0 : 1] += ms;
        }
        spans[r][2] = S.plan.kernels;
    };
    std::vector<int> pending(D, -1);     // the pass whose timing events a set still holds
    for (int r = 0; r < nrep; r++) {
        const int si = r % D;
        ResSet &S = R->set[si];
        if (pending[si] >= 0) {
            // the set's previous pass must be done before its events are reused (engine_run also
            // waits on the stream before it launches)
            if ((e = cudaStreamSynchronize(S.st)) != cudaSuccess) return (int)e;
            read_spans(pending[si], S);
        }
        if (S.exec) {
            // the whole pass, one graph launch, timed as one span
            if ((e = cudaEventRecord(S.tm.ev[0], S.st)) != cudaSuccess) return (int)e;
            if ((e = cudaGraphLaunch(S.exec, S.st)) != cudaSuccess) return (int)e;
            if ((e = cudaEventRecord(S.tm.ev[1], S.st)) != cudaSuccess) return (int)e;
            S.tm.nlaunch = 1;
            S.tm.kind[0] = 2;
        } else {
            const int rc = engine_launch(S.plan, S.d_desc, S.d_list, S.st, &S.tm);
            if (rc != 0) return rc;
        }
        count_launches(S.plan.kernels);
        pending[si] = r;
        R->last = si;
    }
    for (int si = 1; si < D; si++) {
        // each wait takes the record made just before it
        if ((e = cudaEventRecord(R->ev1, R->set[si].st)) != cudaSuccess) return (int)e;
        if ((e = cudaStreamWaitEvent(s0, R->ev1, 0)) != cudaSuccess) return (int)e;
    }
    if ((e = cudaEventRecord(R->ev1, s0)) != cudaSuccess) return (int)e;
    if ((e = cudaEventSynchronize(R->ev1)) != cudaSuccess) return (int)e;
    for (int si = 0; si < D; si++) {
        if ((e = cudaStreamSynchronize(R->set[si].st)) != cudaSuccess) return (int)e;
        if (pending[si] >= 0) read_spans(pending[si], R->set[si]);
    }
    float total = 0.f;
    cudaEventElapsedTime(&total, R->ev0, R->ev1);
    for (int r = 0; r < nrep; r++) {
        times[4 * r] = total / nrep;
        times[4 * r + 1] = spans[r][0];
        times[4 * r + 2] = spans[r][1];
        times[4 * r + 3] = spans[r][2];
    }
    return 0;
}

// results of the last pass back to the problems
int resident_collect(int *ierror) {
    Resident *R = g_res.get();
    if (!R) return -1;
    ResSet &S = R->set[R->last];
    cudaError_t e = cudaMemcpyAsync(R->h_io, S.d_io, R->tot_io, cudaMemcpyDeviceToHost, S.st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(S.st);
    if (e != cudaSuccess) return (int)e;
    for (size_t k = 0; k < R->live.size(); k++) {
        const int i = R->live[k];
        collect(*R->b.probs[i], S.hd[k], (const double *)((const char *)R->h_io + R->off_io[k]));
        ierror[i] = R->b.probs[i]->ierror;
    }
    return 0;
}

// ------------------------------------------------------------------------------------------
// allocation-free solve of one problem.  Some hosts cannot have the library allocate device
// memory once their time loop runs: a multibody code that fixes its device memory budget at
// start-up, or a real-time co-simulation step in which the implicit device synchronisation
// and possible failure of cudaMalloc/cudaFree are not acceptable.  For them every device
// buffer of one solve (descriptor, launch list, io block, work area) is carved from this
// fixed file-scope array; its address is looked up once per device.  Nothing in it has to
// start at zero: the io block is written in full from the host before each solve and the
// solve kernel clears its work columns itself.
// ------------------------------------------------------------------------------------------
constexpr size_t kNoAllocBytes = (size_t)16 << 20;          // 16 MiB: grids up to ~140 x 140
__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];
alignas(256) double g_noalloc_host[kNoAllocBytes / sizeof(double)];   // host staging, no allocation
std::mutex g_noalloc_mu;
constexpr int kMaxDevices = 64;
char *g_noalloc_dev[kMaxDevices] = {};

int calculate_noalloc(int ire, int icp) {
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    Problem *p = lookup(ire, icp, true);
    if (!p) return CNTC_err_icp;
    std::unique_lock<std::mutex> busy(p->busy, std::try_to_lock);
    if (!busy.owns_lock()) return CNTC_err_other;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return CNTC_err_other;
    if (!g_noalloc_dev[dev]) {
        void *addr = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&addr, g_noalloc_scratch);
        if (e != cudaSuccess || !addr) {
            log_msg("cntc_calculate_noalloc: device scratch not available");
            return CNTC_err_other;
        }
        g_noalloc_dev[dev] = (char *)addr;
    }
    auto t0 = std::chrono::steady_clock::now();
    p->ncase++;
    Prep prep;
    int st = prepare(*p, prep);
    if (st != 0) { p->have = false; return st; }
    PatchDesc hd = prep.d;
    if (hd.pvtime == 0 && (hd.tang == 1 || hd.tang == 2) && p->have) {
        // the previous time instance lives in the problem's device copy, which this entry
        // point does not keep
        log_msg("cntc_calculate_noalloc: continuation from the previous time instance (P = 0) is not supported");
        p->have = false;
        return CNTC_err_other;
    }
    const PatchSizes s = patch_sizes(hd.mx, hd.my, hd.fx, hd.fy, hd.nblk, hd.ncf);
    auto up = [](size_t b) { return (b + 255) & ~(size_t)255; };
    const size_t off_list = up(sizeof(PatchDesc)), off_io = off_list + 256, off_work = off_io + up(s.io);
    if (off_work + s.work > kNoAllocBytes || s.io > sizeof(g_noalloc_host)) {
        char msg[160];
        std::snprintf(msg, sizeof msg, "cntc_calculate_noalloc: problem needs %zu bytes of device scratch, limit %zu",
                      off_work + s.work, kNoAllocBytes);
        log_msg(msg);
        p->have = false;
        return CNTC_err_other;
    }
    char *base = g_noalloc_dev[dev];
    carve_patch(hd, base + off_io, base + off_work);
    stage_inputs(*p, hd, g_noalloc_host);
    cudaStream_t stream = cudaStreamPerThread;
    cudaError_t e = cudaMemcpyAsync(base + off_io, g_noalloc_host, s.io, cudaMemcpyHostToDevice, stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(base, &hd, sizeof(PatchDesc), cudaMemcpyHostToDevice, stream);
    if (e != cudaSuccess) { p->have = false; return CNTC_err_other; }
    const unsigned char need_ic = 1;
    int rc = engine_run(&hd, (PatchDesc *)base, 1, &need_ic, (int *)(base + off_list), stream);
    if (rc == 0) e = cudaMemcpyAsync(g_noalloc_host, base + off_io, s.io, cudaMemcpyDeviceToHost, stream);
    if (rc == 0 && e == cudaSuccess) e = cudaStreamSynchronize(stream);
    if (rc != 0 || e != cudaSuccess) { p->have = false; return CNTC_err_other; }
    collect(*p, hd, g_noalloc_host);
    const double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    p->twall += dt; p->tcpu += dt;
    return p->ierror;
}

// ------------------------------------------------------------------------------------------
// serving: cntc_calculate_async / cntc_wait.  Requests go to a queue served by a few worker
// lanes.  A free lane takes every queued request that fits the device-memory admission
// budget and solves them in one engine pass on its own stream; requests that arrive while
// passes are running wait only for the next free lane (continuous batching), and up to
// kLanes passes run on the device at the same time.  Each patch is solved by its own thread
// block, so a result does not depend on which other requests shared its pass.
// ------------------------------------------------------------------------------------------
struct AsyncReq {
    int ire, icp;
    size_t bytes;
    bool done = false;
    int ierror = 0;
    std::chrono::steady_clock::time_point t_submit, t_done;
};

struct Server {
    // a solve keeps its CTA for a long time (seconds for the larger patches), so the device is
    // filled by many passes in flight, not by large ones: up to kLanes passes of at most
    // kMaxPass requests each
    static constexpr int kLanes = 64;
    static constexpr size_t kMaxPass = 16;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<std::shared_ptr<AsyncReq>> queue;
    std::map<long long, std::shared_ptr<AsyncReq>> pending;    // by (ire, icp)
    size_t budget = (size_t)40 << 30;                          // admission budget, bytes
    size_t in_flight = 0;
    std::vector<std::thread> lanes;
    bool stop = false;
    int device = 0;

    void lane_main() {
        cudaSetDevice(device);
        for (;;) {
            std::vector<std::shared_ptr<AsyncReq>> batch;
            size_t bytes = 0;
            {
                std::unique_lock<std::mutex> lk(mu);
                // the problems' device caches (coefficients, previous solutions) count against
                // the budget beside the passes in flight
                auto held = [&] { return in_flight + (size_t)std::max(0LL, g_cache_bytes.load()); };
                cv_work.wait(lk, [&] { return stop || (!queue.empty() && held() + queue.front()->bytes <= budget) ||
                                             (!queue.empty() && in_flight == 0); });
                if (stop && queue.empty()) return;
                while (!queue.empty() && batch.size() < kMaxPass) {
                    const size_t b = queue.front()->bytes;
                    // a single request larger than the budget runs alone
                    if (held() + bytes + b > budget && !(batch.empty() && in_flight == 0)) break;
                    bytes += b;
                    batch.push_back(queue.front());
                    queue.pop_front();
                }
                in_flight += bytes;
            }
            std::vector<int> ire(batch.size()), icp(batch.size()), err(batch.size(), 0);
            for (size_t k = 0; k < batch.size(); k++) { ire[k] = batch[k]->ire; icp[k] = batch[k]->icp; }
            const auto t_start = std::chrono::steady_clock::now();
            // each request completes when its own patch has finished, not at the end of the pass
            std::function<void(int, int)> done = [&](int k, int e) {
                {
                    std::lock_guard<std::mutex> lk(mu);
                    batch[k]->ierror = e;
                    batch[k]->done = true;
                    batch[k]->t_done = std::chrono::steady_clock::now();
                }
                cv_done.notify_all();
            };
            calculate_many((int)batch.size(), ire.data(), icp.data(), err.data(), &done);
            const auto now = std::chrono::steady_clock::now();
            if (g_debug >= 2)
                std::fprintf(stderr, "contact_gb300: serving pass of %zu requests (%.1f MB) took %.3f s\n", batch.size(),
                             bytes / 1e6, std::chrono::duration<double>(now - t_start).count());
            {
                std::lock_guard<std::mutex> lk(mu);
                in_flight -= bytes;
            }
            cv_work.notify_all();
        }
    }

    void ensure_started() {
        if (!lanes.empty()) return;
        cudaGetDevice(&device);
        for (int k = 0; k < kLanes; k++) lanes.emplace_back([this] { lane_main(); });
    }

    ~Server() {
        {
            std::lock_guard<std::mutex> lk(mu);
            stop = true;
        }
        cv_work.notify_all();
        for (auto &t : lanes) if (t.joinable()) t.join();
    }
};

Server &server() {
    static Server s;
    return s;
}

long long pkey2(int ire, int icp) { return (long long)ire * 1000003LL + icp; }

int calculate_async(int ire, int icp) {
    Problem *p = lookup(ire, icp, true);
    if (!p) return CNTC_err_icp;
    Server &S = server();
    auto r = std::make_shared<AsyncReq>();
    r->ire = ire; r->icp = icp;
    const int fx = opt_fft_size(std::max(1, p->mx)), fy = opt_fft_size(std::max(1, p->my));
    const PatchSizes ps = patch_sizes(std::max(1, p->mx), std::max(1, p->my), fx, fy, 1, ncf_of(*p));
    r->bytes = ps.io + ps.work + sizeof(PatchDesc);
    r->t_submit = std::chrono::steady_clock::now();
    {
        std::lock_guard<std::mutex> lk(S.mu);
        const long long key = pkey2(ire, icp);
        // one request per problem at a time, as the reference locks a problem for the duration
        // of a call (m_caddon_data.f90:336-413): a request holds its problem until cntc_wait
        // has returned for it
        if (S.pending.find(key) != S.pending.end()) return CNTC_err_other;
        S.ensure_started();
        S.pending[key] = r;
        S.queue.push_back(r);
    }
    S.cv_work.notify_one();
    return 0;
}

int wait_async(int ire, int icp, double *latency_s) {
    Server &S = server();
    std::unique_lock<std::mutex> lk(S.mu);
    auto it = S.pending.find(pkey2(ire, icp));
    if (it == S.pending.end()) return CNTC_err_icp;
    std::shared_ptr<AsyncReq> r = it->second;
    S.cv_done.wait(lk, [&] { return r->done; });
    S.pending.erase(it);
    if (latency_s) *latency_s = std::chrono::duration<double>(r->t_done - r->t_submit).count();
    return r->ierror;
}

double *field_ptr(Problem &p, int col) {
    const int n = p.r_mx * p.r_my;
    if (!p.have || (int)p.fields.size() < kIoCols * n) return nullptr;
    return p.fields.data() + (size_t)col * n;
}

} // namespace

// ==========================================================================================
// exported functions
// ==========================================================================================
extern "C" {

void cntc_initializefirst(int *ifcver, int *ierror, int *ioutput, const char *c_wrkdir, const char *c_outdir,
                          const char *c_expnam, int *len_wrkdir, int *len_outdir, int *len_expnam) {
    (void)ioutput; (void)c_wrkdir; (void)c_outdir; (void)c_expnam; (void)len_wrkdir; (void)len_outdir; (void)len_expnam;
    g_initialized = 1;
    if (ifcver) *ifcver = kCaddonVersion;
    if (ierror) *ierror = 0;
}

void cntc_initializefirst_new(int *ifcver, int *ierror, int *ioutput, const char *c_wrkdir, const char *c_outdir,
                              const char *c_expnam, int *len_wrkdir, int *len_outdir, int *len_expnam) {
    cntc_initializefirst(ifcver, ierror, ioutput, c_wrkdir, c_outdir, c_expnam, len_wrkdir, len_outdir, len_expnam);
}

void cntc_initialize(int *ire, int *imodul, int *ifcver, int *ierror, const char *c_outdir, int *len_outdir) {
    (void)c_outdir; (void)len_outdir;
    if (g_initialized <= 0) g_initialized = 1;
    if (ifcver) *ifcver = kCaddonVersion;
    if (!ire || *ire <= 0 || *ire > 10000 || !imodul || *imodul != 3) { if (ierror) *ierror = CNTC_err_other; return; }
    if (ierror) *ierror = 0;
}

void cntc_setglobalflags(int *lenflg, int *params, int *values) {
    for (int i = 0; i < *lenflg; i++) {
        if (params[i] == CNTC_if_idebug) g_debug = values[i];
    }
}

void cntc_setflags(int *ire, int *icp, int *lenflg, int *params, int *values) {
    Problem *p = lookup(*ire, *icp, true);
    if (!p) return;
    for (int i = 0; i < *lenflg; i++) {
        const int c = params[i], v = values[i];
        switch (c) {
            case 0: break;
            case CNTC_if_units: select_units(*p, v); break;
            case CNTC_ic_pvtime: p->pvtime = std::max(0, std::min(3, v)); break;
            case CNTC_ic_bound: p->bound = std::max(0, std::min(6, v)); break;
            case CNTC_ic_tang: p->tang = std::max(0, std::min(3, v)); break;
            case CNTC_ic_norm: p->norm = std::max(0, std::min(1, v)); break;
            case CNTC_ic_force: p->force3 = std::max(0, std::min(2, v)); break;
            case CNTC_ic_sens: p->sens = std::max(0, std::min(3, v)); break;
            case CNTC_ic_inflcf: if (v >= 0 && v <= 4) p->gencr = v; break;
            case CNTC_ic_exrhs: p->rztang = std::max(0, std::min(3, v)); break;
            case CNTC_ic_iestim: p->iestim = std::max(0, std::min(3, v)); break;
            case CNTC_ic_matfil: p->matfil = (v < 0 || v > 2) ? 0 : v; break;
            case CNTC_ic_output: p->output = std::max(0, std::min(5, v)); break;
            case CNTC_ic_flow: p->flow = std::max(0, std::min(9, v)); break;
            case CNTC_ic_return: p->ret = std::max(0, std::min(3, v)); break;
            case CNTC_if_ncase: p->ncase = std::max(0, v - 1); break;
            case CNTC_if_mixedprec: p->mixed = (v >= 0 && v <= 4) ? v : 1; break;
            case CNTC_if_groupctas: p->group = (v == -1) ? -1 : std::max(0, v); break;
            default: break;   // output, debugging and module-1 flags have no effect here
        }
    }
}

void cntc_setsolverflags(int *ire, int *icp, int *gdigit, int *nints, int *iparam, int *nreals, double *rparam) {
    static const int nints_loc[7] = {4, 0, 5, 5, 5, 5, 1};
    static const int nreals_loc[7] = {1, 0, 4, 4, 2, 8, 1};
    Problem *p = lookup(*ire, *icp, true);
    if (!p) return;
    const int g = *gdigit;
    if (g < 0 || g > 6) return;
    if (*nints != nints_loc[g] || *nreals != nreals_loc[g]) return;
    if (g != 1 && g != 6) {
        p->gausei_eff = g;
        p->eps = std::max(1e-20, rparam[0]);
        p->maxgs = std::max(1, iparam[0]);
        p->maxin = std::max(1, iparam[1]);
        p->maxnr = std::max(1, iparam[2]);
        p->maxout = std::max(1, iparam[3]);
        if (g == 2 || g == 3) {
            p->inislp = iparam[4];
            p->omegah = std::max(1e-20, rparam[1]);
            p->omegas = std::max(1e-20, rparam[2]);
            p->omgslp = std::max(1e-20, rparam[3]);
        }
        if (g == 4) { p->inislp = iparam[4]; p->omgslp = std::max(1e-20, rparam[1]); }
        if (g == 5) {
            p->fdecay = rparam[1];
            p->betath = rparam[2];
            p->kdowfb = iparam[4];
            p->d_ifc = std::max(0.01, rparam[3]);
            p->d_lin = rparam[4];
            p->d_cns = std::max(0.01, rparam[5]);
            p->d_slp = std::max(0.01, rparam[6]);
            p->pow_s = std::max(0.01, std::min(10.0, rparam[7]));
            if (p->d_lin * (p->d_cns - p->d_ifc) < 0.0) { p->d_lin = 0.0; p->d_cns = p->d_ifc; }
            if (p->fdecay >= 0.999) p->gd_meth = 1;
            else if (p->fdecay <= 0.001) { p->gd_meth = 2; p->kdown = std::max(1, (int)std::lround(-p->fdecay)); }
            else p->gd_meth = 3;
        }
    } else if (g == 6) {
        p->mxsens = std::max(1, iparam[0]);
        p->epsens = std::max(1e-20, rparam[0]);
    }
}

void cntc_setmaterialparameters(int *ire, int *icp, int *imeth, int *nparam, double *rparam) {
    static const int nparam_loc[13] = {4, 8, 8, 7, 8, 7, 4, 4, 0, 0, 0, 0, 4};
    Problem *p = lookup(*ire, *icp, true);
    if (!p) return;
    const int m = *imeth;
    const bool set_m = m >= 0 && m <= 7, set_m2 = m >= 10 && m <= 12;
    if (!set_m && !set_m2) return;
    if ((nparam_loc[m] == 0 && *nparam >= 2) || (nparam_loc[m] != 0 && *nparam != nparam_loc[m])) return;
    if (set_m2) return;     // damping (M2 digit) does not change the solve
    p->mater = m;
    p->poiss[0] = rparam[0]; p->poiss[1] = rparam[1];
    p->gg[0] = rparam[2] * p->s_forc / p->s_area;
    p->gg[1] = rparam[3] * p->s_forc / p->s_area;
    // MAXOUT for quasi-identical and other material pairs (src/contact_addon.f90:1458-1462)
    const double ga = 2.0 / (1.0 / p->gg[0] + 1.0 / p->gg[1]);
    const double ak = (ga / 4.0) * ((1.0 - 2.0 * p->poiss[0]) / p->gg[0] - (1.0 - 2.0 * p->poiss[1]) / p->gg[1]);
    if (p->maxout >= 2 && std::fabs(ak) < 1e-4) p->maxout = 1;
    if (p->maxout <= 1 && std::fabs(ak) >= 1e-4) p->maxout = 10;
}

// H digit (cntc_setTemperatureData, src/contact_addon.f90:1477-1550): the method is recorded
// so that a solve with temperatures (H = 3) is refused; the temperature data are not used
void cntc_settemperaturedata(int *ire, int *icp, int *imeth, int *nparam, double *rparam) {
    (void)rparam;
    static const int nparam_loc[4] = {0, 0, 0, 9};
    Problem *p = lookup(*ire, *icp, true);
    if (!p) return;
    const int h = *imeth;
    if (h < 0 || h == 2 || h > 3) return;
    if ((nparam_loc[h] == 0 && *nparam >= 2) || (nparam_loc[h] != 0 && *nparam != nparam_loc[h])) return;
    p->heat = h;
}

void cntc_settimestep(int *ire, int *icp, double *dt) {
    Problem *p = lookup(*ire, *icp, true);
    if (p) p->dt = *dt;
}

void cntc_setreferencevelocity(int *ire, int *icp, double *veloc) {
    Problem *p = lookup(*ire, *icp, true);
    if (p) p->veloc = std::max(1e-9, std::fabs(*veloc) * p->s_veloc);
}

void cntc_setrollingstepsize(int *ire, int *icp, double *chi, double *dq) {
    Problem *p = lookup(*ire, *icp, true);
    if (!p) return;
    p->chi = *chi * p->s_angle;
    p->dq = *dq * p->s_len;
}

void cntc_setfrictionmethod(int *ire, int *icp, int *imeth, int *nparam, double *params) {
    static const int nparam_loc[7] = {2, 0, 7, 7, 7, 3, 6};
    Problem *p = lookup(*ire, *icp, true);
    if (!p) return;
    const int vdigit = *imeth / 10, ldigit = *imeth - 10 * vdigit;
    if (vdigit < 0 || vdigit > 2 || ldigit < 0 || ldigit > 6) return;
    if (ldigit == 1) return;
    if (vdigit != 0) { p->varfrc = vdigit; return; }
    if (*nparam != nparam_loc[ldigit]) return;
    p->varfrc = 0;
    p->frclaw = (ldigit == 5) ? 4 : ldigit;
    if (ldigit == 0) {
        p->fkin = std::max(1e-6, std::min(params[0], params[1]));
        p->fstat = p->fkin;
        p->muscal = p->fstat;
    }
}

void cntc_sethertzcontact(int *ire, int *icp, int *ipotcn, int *nparam, double *params) {
    static const int nparam_loc[6] = {6, 5, 5, 5, 5, 5};
    Problem *p = lookup(*ire, *icp, true);
    if (!p) return;
    const int ip = *ipotcn;
    if (ip < -6 || ip > -1 || *nparam != nparam_loc[ip + 6]) return;
    p->ipotcn = ip;
    p->mx = std::max(1, (int)std::lround(params[0]));
    p->my = std::max(1, (int)std::lround(params[1]));
    if (ip == -3) {
        p->hz_aa = std::max(1e-6, params[2]) * p->s_len;
        p->hz_bb = std::max(1e-6, params[3]) * p->s_len;
        p->hz_scale = std::max(1e-6, params[4]);
    } else if (ip == -2) {
        p->hz_a1 = std::max(1e-12, params[2]) / p->s_len;
        p->hz_aob = std::max(1e-6, params[3]);
        p->hz_scale = std::max(1e-6, params[4]);
    } else if (ip == -1) {
        p->hz_a1 = std::max(1e-12, params[2]) / p->s_len;
        p->hz_b1 = std::max(1e-12, params[3]) / p->s_len;
        p->hz_scale = std::max(1e-6, params[4]);
    } else {
        p->ipotcn = ip;   // 2-D and SDEC variants are stored but not solved by this engine
    }
}

void cntc_setpotcontact(int *ire, int *icp, int *ipotcn, int *nparam, double *params) {
    Problem *p = lookup(*ire, *icp, true);
    if (!p) return;
    const int ip = *ipotcn;
    if (ip < 1 || ip > 4 || *nparam != 6) return;
    p->ipotcn = ip;
    p->mx = std::max(1, (int)std::lround(params[0]));
    p->my = std::max(1, (int)std::lround(params[1]));
    const double a = params[2] * p->s_len, b = params[3] * p->s_len;
    // potcon_fill, m_hierarch_data.f90:1801-1861
    if (ip == 1) { p->xl = a; p->yl = b; p->dx = std::max(1e-12, params[4]) * p->s_len; p->dy = std::max(1e-12, params[5]) * p->s_len; }
    else if (ip == 2) { p->xl = a; p->yl = b; p->dx = (params[4] * p->s_len - a) / p->mx; p->dy = (params[5] * p->s_len - b) / p->my; }
    else if (ip == 3) {
        p->dx = std::max(1e-12, params[4]) * p->s_len; p->dy = std::max(1e-12, params[5]) * p->s_len;
        p->xl = a - 0.5 * p->dx; p->yl = b - 0.5 * p->dy;
    } else {
        p->dx = (params[4] * p->s_len - a) / std::max(1, p->mx - 1);
        p->dy = (params[5] * p->s_len - b) / std::max(1, p->my - 1);
        p->xl = a - 0.5 * p->dx; p->yl = b - 0.5 * p->dy;
    }
}

void cntc_setpenetration(int *ire, int *icp, double *pen) {
    Problem *p = lookup(*ire, *icp, true);
    if (!p) return;
    p->norm = 0;
    p->pen = *pen * p->s_len;
}

void cntc_setnormalforce(int *ire, int *icp, double *fn) {
    Problem *p = lookup(*ire, *icp, true);
    if (!p) return;
    p->norm = 1;
    p->fn = *fn;
}

void cntc_setundeformeddistc(int *ire, int *icp, int *ibase, int *nparam, double *prmudf) {
    Problem *p = lookup(*ire, *icp, true);
    if (!p) return;
    const int ib = *ibase;
    int need;
    if (ib == 1) need = 6;
    else if (ib == 9) need = p->mx * p->my;
    else return;      // ibase 2, 3 are not provided by this engine
    if (*nparam != need) return;
    p->ibase = ib;
    if (ib == 1) {
        p->prmudf.assign(6, 0.0);
        for (int k = 0; k < 3; k++) p->prmudf[k] = prmudf[k] / p->s_len;
        for (int k = 3; k < 5; k++) p->prmudf[k] = prmudf[k];
        p->prmudf[5] = prmudf[5] * p->s_len;
    } else {
        p->prmudf.assign(prmudf, prmudf + need);
        for (auto &v : p->prmudf) v *= p->s_len;
    }
}

void cntc_setcreepages(int *ire, int *icp, double *vx, double *vy, double *phi) {
    Problem *p = lookup(*ire, *icp, true);
    if (!p) return;
    if (p->tang == 1) { p->cksi = *vx * p->s_len; p->ceta = *vy * p->s_len; p->cphi = *phi; }
    else { p->cksi = *vx; p->ceta = *vy; p->cphi = *phi / p->s_len; }
}

void cntc_setextrarigidslip(int *ire, int *icp, int *lenarr, double *wx, double *wy) {
    (void)lenarr; (void)wx; (void)wy;
    Problem *p = lookup(*ire, *icp, true);
    if (p) p->rztang = 1;   // stored as a request; the solve reports it as unsupported
}

void cntc_settangentialforces(int *ire, int *icp, double *fx, double *fy) {
    Problem *p = lookup(*ire, *icp, true);
    if (!p) return;
    p->fxrel = *fx; p->fyrel = *fy;
    const double fabs_ = std::sqrt((*fx) * (*fx) + (*fy) * (*fy));
    if (fabs_ > 1.0) { p->fxrel /= fabs_; p->fyrel /= fabs_; }
}

void cntc_calculate(int *ire, int *icp, int *ierror) {
    int ie = 0;
    calculate_many(1, ire, icp, &ie);
    *ierror = ie;
}

void cntc_calculate_async(int *ire, int *icp, int *ierror) {
    *ierror = calculate_async(*ire, *icp);
}

void cntc_wait(int *ire, int *icp, int *ierror) {
    *ierror = wait_async(*ire, *icp, nullptr);
}

void cntc_gb300_wait_latency(int *ire, int *icp, int *ierror, double *latency) {
    *ierror = wait_async(*ire, *icp, latency);
}

void cntc_gb300_setadmissionbudget(double *gbytes) {
    Server &S = server();
    std::lock_guard<std::mutex> lk(S.mu);
    S.budget = (size_t)(std::max(0.0, *gbytes) * 1e9);
}

void cntc_calculate_noalloc(int *ire, int *icp, int *ierror) {
    *ierror = calculate_noalloc(*ire, *icp);
}

void cntc_calculate_batch(int *n, int *ire, int *icp, int *ierror) {
    if (!n || *n <= 0) return;
    calculate_many(*n, ire, icp, ierror);
}

void cntc_getflags(int *ire, int *icp, int *lenflg, int *params, int *values) {
    Problem *p = lookup(*ire, *icp, false);
    for (int i = 0; i < *lenflg; i++) {
        int v = 0;
        if (p) {
            switch (params[i]) {
                case CNTC_if_units: v = p->units; break;
                case CNTC_ic_pvtime: v = p->pvtime; break;
                case CNTC_ic_bound: v = p->bound; break;
                case CNTC_ic_tang: v = p->tang; break;
                case CNTC_ic_norm: v = p->norm; break;
                case CNTC_ic_force: v = p->force3; break;
                case CNTC_ic_frclaw: v = p->frclaw; break;
                case CNTC_ic_mater: v = p->mater; break;
                case CNTC_ic_iestim: v = p->iestim; break;
                case CNTC_if_ncase: v = p->ncase; break;
                case CNTC_if_mixedprec: v = p->mixed; break;
                case CNTC_if_groupctas: v = p->group; break;
                default: v = 0;
            }
        }
        values[i] = v;
    }
}

void cntc_gethertzcontact(int *ire, int *icp, int *lenarr, double *rvalues) {
    Problem *p = lookup(*ire, *icp, false);
    if (!p) return;
    const double v[10] = {p->hz_a1 * p->s_len, p->hz_b1 * p->s_len, p->hz_aa / p->s_len, p->hz_bb / p->s_len,
                          p->hz_rho / p->s_len, p->hz_cp / p->s_len, p->hz_scale, 0.0, 0.0, p->hz_aob};
    for (int i = 0; i < *lenarr && i < 10; i++) rvalues[i] = v[i];
}

void cntc_getnumelements(int *ire, int *icp, int *mx, int *my) {
    Problem *p = lookup(*ire, *icp, false);
    if (!p) return;
    *mx = p->have ? p->r_mx : p->mx;
    *my = p->have ? p->r_my : p->my;
}

void cntc_getgriddiscretization(int *ire, int *icp, double *dx, double *dy) {
    Problem *p = lookup(*ire, *icp, false);
    if (!p) return;
    *dx = p->r_dx / p->s_len;
    *dy = p->r_dy / p->s_len;
}

void cntc_getpotcontact(int *ire, int *icp, int *lenarr, double *rvalues) {
    Problem *p = lookup(*ire, *icp, false);
    if (!p) return;
    const double v[6] = {(double)p->r_mx, (double)p->r_my, p->r_xc1 / p->s_len, p->r_yc1 / p->s_len,
                         p->r_dx / p->s_len, p->r_dy / p->s_len};
    for (int i = 0; i < *lenarr; i++) rvalues[i] = i < 6 ? v[i] : 0.0;
}

void cntc_getpenetration(int *ire, int *icp, double *pen) {
    Problem *p = lookup(*ire, *icp, false);
    if (p) *pen = p->pen / p->s_len;
}

void cntc_getcreepages(int *ire, int *icp, double *vx, double *vy, double *phi) {
    Problem *p = lookup(*ire, *icp, false);
    if (!p) return;
    if (p->tang == 1) { *vx = p->s_body * p->cksi / p->s_len; *vy = p->s_body * p->ceta / p->s_len; *phi = p->s_body * p->cphi; }
    else { *vx = p->s_body * p->cksi; *vy = p->s_body * p->ceta; *phi = p->s_body * p->cphi * p->s_len; }
}

void cntc_getreferencevelocity(int *ire, int *icp, double *veloc) {
    Problem *p = lookup(*ire, *icp, false);
    if (p) *veloc = p->veloc / p->s_veloc;
}

void cntc_getcontactforces(int *ire, int *icp, double *fn, double *tx, double *ty, double *mz) {
    Problem *p = lookup(*ire, *icp, false);
    if (!p) return;
    *fn = p->f_n;
    *tx = p->s_body * p->f_x;
    *ty = p->s_body * p->f_y;
    *mz = p->s_body * p->m_z / p->s_len;
}

void cntc_getcontactpatchareas(int *ire, int *icp, double *carea, double *harea, double *sarea) {
    Problem *p = lookup(*ire, *icp, false);
    if (!p) return;
    const double dxdy = p->r_dx * p->r_dy;
    *carea = (double)(float)p->ncon * dxdy / p->s_area;
    *harea = (double)(float)p->nadh * dxdy / p->s_area;
    *sarea = (double)(float)p->nslip * dxdy / p->s_area;
}

void cntc_getelementdivision(int *ire, int *icp, int *lenarr, int *eldiv) {
    Problem *p = lookup(*ire, *icp, false);
    if (!p || !p->have) return;
    const int n = std::min(*lenarr, (int)p->igs.size());
    for (int i = 0; i < n; i++) eldiv[i] = p->igs[i];
}

void cntc_getmaximumpressure(int *ire, int *icp, double *pnmax) {
    Problem *p = lookup(*ire, *icp, false);
    if (!p) return;
    const double *pn = field_ptr(*p, W_PN);
    double m = 0.0;
    if (pn) for (int i = 0; i < p->r_mx * p->r_my; i++) m = std::max(m, std::fabs(pn[i]));
    *pnmax = m * p->s_area;
}

void cntc_getmaximumtraction(int *ire, int *icp, double *ptmax) {
    Problem *p = lookup(*ire, *icp, false);
    if (!p) return;
    const double *px = field_ptr(*p, W_PX), *py = field_ptr(*p, W_PY);
    double m = -1.0;
    if (px) for (int i = 0; i < p->r_mx * p->r_my; i++) m = std::max(m, std::sqrt(px[i] * px[i] + py[i] * py[i]));
    *ptmax = m * p->s_area;
}

void cntc_getfielddata(int *ire, int *icp, int *ifld, int *lenarr, double *fld) {
    Problem *p = lookup(*ire, *icp, false);
    if (!p || !p->have) return;
    const int n = p->r_mx * p->r_my;
    int col = -1;
    double sc = 1.0;
    std::vector<double> tmp;
    const double *src = nullptr;
    switch (*ifld) {
        case CNTC_fld_h: col = W_H; sc = 1.0 / p->s_len; break;
        case CNTC_fld_mu: tmp.assign(n, p->fstat); src = tmp.data(); break;
        case CNTC_fld_px: col = W_PX; sc = p->s_area * p->s_body; break;
        case CNTC_fld_py: col = W_PY; sc = p->s_area * p->s_body; break;
        case CNTC_fld_pn: col = W_PN; sc = p->s_area; break;
        case CNTC_fld_ux: col = W_UX; sc = 1.0 / p->s_len; break;
        case CNTC_fld_uy: col = W_UY; sc = 1.0 / p->s_len; break;
        case CNTC_fld_un: col = W_UN; sc = 1.0 / p->s_len; break;
        case CNTC_fld_sx: col = W_SX; sc = p->s_body / p->r_dq; break;
        case CNTC_fld_sy: col = W_SY; sc = p->s_body / p->r_dq; break;
        case CNTC_fld_wx: col = W_WX; sc = p->s_body / p->r_dq; break;
        case CNTC_fld_wy: col = W_WY; sc = p->s_body / p->r_dq; break;
        case CNTC_fld_taucrt: case CNTC_fld_uplsx: case CNTC_fld_uplsy: case CNTC_fld_temp1: case CNTC_fld_temp2:
            tmp.assign(n, 0.0); src = tmp.data(); break;
        default: return;
    }
    if (col >= 0) src = field_ptr(*p, col);
    if (!src) return;
    for (int i = 0; i < n && i < *lenarr; i++) fld[i] = sc * src[i];
}

void cntc_gettractions(int *ire, int *icp, int *lenarr, double *pn, double *px, double *py) {
    int f;
    f = CNTC_fld_px; cntc_getfielddata(ire, icp, &f, lenarr, px);
    f = CNTC_fld_py; cntc_getfielddata(ire, icp, &f, lenarr, py);
    f = CNTC_fld_pn; cntc_getfielddata(ire, icp, &f, lenarr, pn);
}

void cntc_getmicroslip(int *ire, int *icp, int *lenarr, double *sx, double *sy) {
    int f;
    f = CNTC_fld_sx; cntc_getfielddata(ire, icp, &f, lenarr, sx);
    f = CNTC_fld_sy; cntc_getfielddata(ire, icp, &f, lenarr, sy);
}

void cntc_getdisplacements(int *ire, int *icp, int *lenarr, double *un, double *ux, double *uy) {
    int f;
    f = CNTC_fld_ux; cntc_getfielddata(ire, icp, &f, lenarr, ux);
    f = CNTC_fld_uy; cntc_getfielddata(ire, icp, &f, lenarr, uy);
    f = CNTC_fld_un; cntc_getfielddata(ire, icp, &f, lenarr, un);
}

// sens(iout + (iin-1) lenout) for outputs fn, fx, fy, mz and inputs pen, cksi, ceta, cphi, in the
// caller's units (cntc_getSensitivities 5919-6007): zero where not computed.  The Newton-Raphson on
// prescribed total forces leaves d(Fx, Fy)/d(cksi, ceta); S >= 2 adds dFn/dpen, S >= 3 the
// derivatives of Fx, Fy and Mz with respect to all three creepages.
void cntc_getsensitivities(int *ire, int *icp, int *lenout, int *lenin, double *sens) {
    for (int i = 0; i < (*lenout) * (*lenin); i++) sens[i] = 0.0;
    Problem *p = lookup(*ire, *icp, false);
    if (!p) return;
    // internal -> external: d out / d in * fac_in / fac_out (module 3: no mirroring)
    double fac_in[4] = {p->s_len, 1.0, 1.0, 1.0 / p->s_len};
    if (p->tang == 1) { fac_in[1] = p->s_len; fac_in[2] = p->s_len; fac_in[3] = 1.0; }
    const double fac_out[4] = {p->s_forc, 1.0, 1.0, p->s_forc * p->s_len};
    for (int iin = 1; iin <= *lenin; iin++)
        for (int iout = 1; iout <= *lenout; iout++)
            if (iout <= 4 && iin <= 4)
                sens[(iout - 1) + (iin - 1) * (*lenout)] =
                    p->sens_all[(iout - 1) * 4 + (iin - 1)] * fac_in[iin - 1] / fac_out[iout - 1];
}

void cntc_getcalculationtime(int *ire, int *icp, double *tcpu, double *twall) {
    Problem *p = lookup(*ire, *icp, false);
    if (!p) { *tcpu = 0; *twall = 0; return; }
    *tcpu = p->tcpu; *twall = p->twall;
}

void cntc_resetcalculationtime(int *ire, int *icp) {
    Problem *p = lookup(*ire, *icp, false);
    if (p) { p->tcpu = 0; p->twall = 0; }
}

void cntc_getiterationcounts(int *ire, int *icp, int *lenarr, int *values) {
    Problem *p = lookup(*ire, *icp, false);
    if (!p) return;
    const int v[6] = {p->itnorm, p->ittang, p->itcg, p->itgs, p->solver, p->ierror};
    for (int i = 0; i < *lenarr && i < 6; i++) values[i] = v[i];
}

void cntc_getparameters(int *ire, int *icp, int *itask, int *lenarr, double *values) {
    Problem *p = lookup(*ire, *icp, false);
    if (!p) return;
    const int n = *lenarr;
    auto put = [&](int k, double v) { if (k <= n) values[k - 1] = v; };
    if (*itask == 1) {
        put(1, p->veloc / p->s_veloc);
        put(2, p->chi / p->s_angle);
        put(3, (p->have ? p->r_dq : p->dq) / p->s_len);
        put(4, 0.0); put(5, 0.0);            // spin centre offsets: not supported, zero
        put(6, 0.0);                         // tau_c0: elastic material
    } else if (*itask == 2) {
        // combin_mater (m_hierarch_data.f90:1543-1553)
        const double ga = 2.0 / (1.0 / p->gg[0] + 1.0 / p->gg[1]);
        const double nu = ga * (p->poiss[0] / p->gg[0] + p->poiss[1] / p->gg[1]) / 2.0;
        const double ak = (ga / 4.0) * ((1.0 - 2.0 * p->poiss[0]) / p->gg[0] - (1.0 - 2.0 * p->poiss[1]) / p->gg[1]);
        put(1, p->gg[0] * p->s_area); put(2, p->gg[1] * p->s_area); put(3, ga * p->s_area);
        put(4, p->poiss[0]); put(5, p->poiss[1]); put(6, nu); put(7, ak);
        for (int k = 8; k <= 22; k++) put(k, 0.0);   // no flexibility, layer, damping or plasticity data
    } else if (*itask == 3) {
        put(1, 0.0);                         // Coulomb friction (L = 0)
        put(2, 1.0); put(3, 0.0); put(4, 0.0);
        put(5, 0.0); put(6, p->fstat); put(7, p->fkin);
    }
}

void cntc_setmetadata(int *ire, int *icp, int *lenmta, int *params, double *values) {
    (void)ire; (void)icp; (void)lenmta; (void)params; (void)values;   // output metadata only
}

void cntc_getmaximumtemperature(int *ire, int *icp, double *t1max, double *t2max) {
    if (!lookup(*ire, *icp, false)) return;
    *t1max = 0.0;
    *t2max = 0.0;
}

// outside the solve path: wheel-rail module, input-file reader, subsurface stresses
static void not_supported(const char *name) {
    char msg[160];
    std::snprintf(msg, sizeof msg, "%s: not supported by this library (module-3 solve path only)", name);
    log_msg(msg);
}
static void zero(int *lenarr, double *values) { for (int i = 0; i < *lenarr; i++) values[i] = 0.0; }

void cntc_readinpfile(int *, int *, const char *, int *, int *ierror) {
    not_supported("cntc_readinpfile");
    *ierror = CNTC_err_other;
}
void cntc_setverticalforce(int *, double *) { not_supported("cntc_setverticalforce"); }
void cntc_setprofileinputfname(int *, const char *, int *, int *, int *, int *, double *) {
    not_supported("cntc_setprofileinputfname");
}
void cntc_setprofileinputvalues(int *, int *, double *, int *, int *, int *, double *) {
    not_supported("cntc_setprofileinputvalues");
}
void cntc_settrackdimensions(int *, int *, int *, double *) { not_supported("cntc_settrackdimensions"); }
void cntc_setwheelsetdimensions(int *, int *, int *, double *) { not_supported("cntc_setwheelsetdimensions"); }
void cntc_setwheelsetposition(int *, int *, int *, double *) { not_supported("cntc_setwheelsetposition"); }
void cntc_setwheelsetvelocity(int *, int *, int *, double *) { not_supported("cntc_setwheelsetvelocity"); }
void cntc_setwheelsetflexibility(int *, int *, int *, double *) { not_supported("cntc_setwheelsetflexibility"); }
void cntc_getprofilevalues(int *, int *, int *, int *, int *, double *, int *lenarr, double *values) {
    not_supported("cntc_getprofilevalues");
    zero(lenarr, values);
}
void cntc_getprofilevalues_new(int *, int *, int *, int *, int *, double *, int *lenarr, double *values) {
    not_supported("cntc_getprofilevalues_new");
    zero(lenarr, values);
}
void cntc_getwheelsetposition(int *, int *lenarr, double *values) {
    not_supported("cntc_getwheelsetposition");
    zero(lenarr, values);
}
void cntc_getwheelsetvelocity(int *, int *lenarr, double *values) {
    not_supported("cntc_getwheelsetvelocity");
    zero(lenarr, values);
}
void cntc_getnumcontactpatches(int *, int *npatch) {
    not_supported("cntc_getnumcontactpatches");
    *npatch = 0;
}
void cntc_getcontactlocation(int *, int *, int *lenarr, double *values) {
    not_supported("cntc_getcontactlocation");
    zero(lenarr, values);
}
void cntc_getglobalforces(int *, int *, int *lenarr, double *values) {
    not_supported("cntc_getglobalforces");
    zero(lenarr, values);
}
// ------------------------------------------------------------------------------------------
// subsurface stresses (module 3): subs_addBlock 3330-3515, subs_calculate 3904-3997,
// subs_getBlocksize 6071-6109, subs_getResults 6113-6187 of src/contact_addon.f90
// ------------------------------------------------------------------------------------------
constexpr int kMaxSubsBlocks = 10, kMaxSubsPoints = 9999;      // MXBLCK, MXSUBS (m_globals.f90:32-33)

void subs_addblock(int *ire, int *icp, int *iblk, int *isubs, int *npx, int *npy, int *npz, double *xparam,
                   double *yparam, double *zparam) {
    static const int npx_loc[10] = {0, 0, 3, -1, 0, 0, 3, -1, 0, -1}, npz_loc[10] = {0, 3, 3, 3, 0, -1, -1, -1, 0, -1};
    Problem *p = lookup(*ire, *icp, true);
    if (!p) return;
    const int t = *isubs, b = *iblk;
    if (b < 0 || b > std::min(kMaxSubsBlocks, (int)p->subs.size() + 1)) { log_msg("subs_addblock: invalid block"); return; }
    if (t < 1 || t == 4 || t == 8 || t > 9) { log_msg("subs_addblock: block type does not exist"); return; }
    if ((npx_loc[t] > 0 && *npx != npx_loc[t]) || (npx_loc[t] > 0 && *npy != npx_loc[t]) ||
        (npz_loc[t] > 0 && *npz != npz_loc[t])) {
        log_msg("subs_addblock: wrong number of parameters for the block type");
        return;
    }
    // blocks iblk and higher are replaced; iblk <= 0 clears the list
    p->subs.resize(std::max(0, b - 1));
    if (b <= 0) return;
    SubsBlock s;
    s.isubs = t;
    // a list of n <= 0 values is empty (its array is not read): the block then has no points
    auto clamp_n = [](int n) { return std::max(0, std::min(n, kMaxSubsPoints)); };
    auto unique_positive = [&](int n, const double *v) {
        std::vector<int> r;
        for (int i = 0; i < clamp_n(n); i++) { const int k = (int)std::lround(v[i]); if (k > 0) r.push_back(k); }
        std::sort(r.begin(), r.end());
        r.erase(std::unique(r.begin(), r.end()), r.end());
        return r;
    };
    if (t == 2 || t == 6) {
        s.ixl = std::max((int)std::lround(xparam[0]), 1);
        s.ixinc = std::max((int)std::lround(xparam[1]), 1);
        s.ixh = std::min((int)std::lround(xparam[2]), 999999);
        s.iyl = std::max((int)std::lround(yparam[0]), 1);
        s.iyinc = std::max((int)std::lround(yparam[1]), 1);
        s.iyh = std::min((int)std::lround(yparam[2]), 999999);
    } else if (t == 3 || t == 7) {
        s.ixlist = unique_positive(*npx, xparam);
        s.iylist = unique_positive(*npy, yparam);
    }
    if (t >= 1 && t <= 3) {
        s.nz = clamp_n((int)std::lround(zparam[0]));
        s.zl = zparam[1] * p->s_len;
        s.dz = std::max(zparam[2] * p->s_len, 1e-9);
    } else {
        s.nz = clamp_n(*npz);
        s.z.assign(zparam, zparam + s.nz);
        for (double &v : s.z) v *= p->s_len;
        std::sort(s.z.begin(), s.z.end());
    }
    if (t == 9) {
        s.x.assign(xparam, xparam + clamp_n(*npx));
        s.y.assign(yparam, yparam + clamp_n(*npy));
        for (double &v : s.x) v *= p->s_len;
        for (double &v : s.y) v *= p->s_len;
        std::sort(s.x.begin(), s.x.end());
        std::sort(s.y.begin(), s.y.end());
    }
    p->subs.push_back(s);
}

// one block (expand_xb, m_subsurf.f90:440-620, then the field at its points): element centres
// depth by depth, explicit points in one pass
static int subs_block(const Problem &p, SubsBlock &s) {
    const int mx = p.r_mx, my = p.r_my, n = mx * my;
    std::vector<int> ixs, iys;
    std::vector<double> xs, ys;
    if (s.isubs == 9) {
        xs = s.x; ys = s.y;
    } else {
        if (s.isubs == 3 || s.isubs == 7) {
            for (int k : s.ixlist) if (k >= 1 && k <= mx) ixs.push_back(k);
            for (int k : s.iylist) if (k >= 1 && k <= my) iys.push_back(k);
        } else {
            for (int k = std::max(s.ixl, 1); k <= std::min(s.ixh, mx); k += s.ixinc) ixs.push_back(k);
            for (int k = std::max(s.iyl, 1); k <= std::min(s.iyh, my); k += s.iyinc) iys.push_back(k);
        }
        for (int k : ixs) xs.push_back(p.r_xc1 + (double)(float)(k - 1) * p.r_dx);
        for (int k : iys) ys.push_back(p.r_yc1 + (double)(float)(k - 1) * p.r_dy);
    }
    std::vector<double> zs = s.z;
    if (s.isubs >= 1 && s.isubs <= 3) {
        zs.resize(s.nz);
        for (int k = 0; k < s.nz; k++) zs[k] = s.zl + (double)(float)k * s.dz;
    }
    s.nx_eff = (int)xs.size(); s.ny_eff = (int)ys.size();
    const int nxy = s.nx_eff * s.ny_eff, nz = (int)zs.size(), npt = nxy * nz;
    s.table.assign((size_t)npt * 21, 0.0);
    if (npt == 0) return 0;
    cgb::SubsLoad L;
    L.mx = mx; L.my = my; L.dx = p.r_dx; L.dy = p.r_dy; L.xc1 = p.r_xc1; L.yc1 = p.r_yc1;
    L.pn = p.fields.data() + (size_t)W_PN * n;
    L.px = p.fields.data() + (size_t)W_PX * n;
    L.py = p.fields.data() + (size_t)W_PY * n;
    L.gg[0] = p.gg[0]; L.gg[1] = p.gg[1]; L.poiss[0] = p.poiss[0]; L.poiss[1] = p.poiss[1];
    std::vector<double> res((size_t)npt * cgb::kSubsCols);
    int rc = 0;
    if (s.isubs == 9) {
        std::vector<double> xyz((size_t)npt * 3);
        for (int iz = 0, q = 0; iz < nz; iz++)
            for (int iy = 0; iy < s.ny_eff; iy++)
                for (int ix = 0; ix < s.nx_eff; ix++, q++) {
                    xyz[3 * q] = xs[ix]; xyz[3 * q + 1] = ys[iy]; xyz[3 * q + 2] = zs[iz];
                }
        rc = cgb::subs_points(L, npt, xyz.data(), res.data());
    } else {
        for (int iz = 0; iz < nz && rc == 0; iz++)
            rc = cgb::subs_depth(L, zs[iz], s.nx_eff, ixs.data(), s.ny_eff, iys.data(),
                                 res.data() + (size_t)iz * nxy * cgb::kSubsCols);
    }
    if (rc != 0) return rc;
    for (int iz = 0, q = 0; iz < nz; iz++)
        for (int iy = 0; iy < s.ny_eff; iy++)
            for (int ix = 0; ix < s.nx_eff; ix++, q++) {
                double *row = s.table.data() + (size_t)q * 21;
                const double *o = res.data() + (size_t)q * cgb::kSubsCols;
                row[0] = xs[ix]; row[1] = ys[iy]; row[2] = zs[iz];
                for (int c = 0; c < 9; c++) row[3 + c] = o[c];
                // the stress tensor by columns: sigxx, sigyx, sigzx, sigxy, ...
                for (int j = 0; j < 3; j++)
                    for (int i = 0; i < 3; i++) row[12 + i + 3 * j] = o[9 + 3 * i + j];
            }
    return 0;
}

void subs_calculate(int *ire, int *icp, int *ierror) {
    *ierror = 0;
    Problem *p = lookup(*ire, *icp, true);
    if (!p) { *ierror = CNTC_err_icp; return; }
    std::unique_lock<std::mutex> lk(p->busy, std::try_to_lock);
    if (!lk.owns_lock()) { *ierror = CNTC_err_other; return; }
    // the tractions of the last solve on its grid (the reference takes the problem's current
    // output without a check; here a problem without a solution is refused)
    if (!p->have || (int)p->fields.size() < kIoCols * p->r_mx * p->r_my) {
        log_msg("subs_calculate: no solution to evaluate");
        *ierror = CNTC_err_other;
        return;
    }
    for (SubsBlock &s : p->subs) {
        const int rc = subs_block(*p, s);
        if (rc != 0) {
            if (g_debug >= 1) std::fprintf(stderr, "contact_gb300: subsurface error %d\n", rc);
            *ierror = CNTC_err_other;
            return;
        }
    }
}

void subs_getblocksize(int *ire, int *icp, int *iblk, int *nx, int *ny, int *nz) {
    *nx = 0; *ny = 0; *nz = 0;
    Problem *p = lookup(*ire, *icp, false);
    if (!p || *iblk <= 0 || *iblk > (int)p->subs.size()) return;
    const SubsBlock &s = p->subs[*iblk - 1];
    if (s.table.empty() && s.nx_eff * s.ny_eff == 0) return;
    *nx = s.nx_eff; *ny = s.ny_eff;
    *nz = (s.nx_eff * s.ny_eff > 0) ? (int)(s.table.size() / 21) / (s.nx_eff * s.ny_eff) : 0;
}

void subs_getresults(int *ire, int *icp, int *iblk, int *lenarr, int *ncol, int *icol, double *values) {
    Problem *p = lookup(*ire, *icp, false);
    if (!p || *iblk <= 0 || *iblk > (int)p->subs.size()) return;
    const SubsBlock &s = p->subs[*iblk - 1];
    const int npnt = (int)(s.table.size() / 21);
    for (int jc = 0; jc < *ncol; jc++) {
        double *out = values + (size_t)jc * std::max(0, *lenarr);
        const int c = icol[jc];
        if (c <= 0 || c > 21) { for (int i = 0; i < *lenarr; i++) out[i] = -999.0; continue; }
        // lengths and displacements in the caller's length unit, stresses in its stress unit
        const double f = c <= 6 ? 1.0 / p->s_len : p->s_area / p->s_forc;
        for (int i = 0; i < std::min(npnt, *lenarr); i++) out[i] = s.table[(size_t)i * 21 + (c - 1)] * f;
    }
}

void cntc_finalize(int *ire) {
    std::lock_guard<std::mutex> lk(g_mu);
    for (auto it = g_problems.begin(); it != g_problems.end();) {
        if (it->second->ire == *ire) { it->second->release_device(); it = g_problems.erase(it); }
        else ++it;
    }
}

void cntc_finalizelast() {
    std::lock_guard<std::mutex> lk(g_mu);
    for (auto &kv : g_problems) kv.second->release_device();
    g_problems.clear();
    g_initialized = -1;
}

long long cntc_gb300_kernel_launches() { return cgb::kernel_launch_count(); }

void cntc_gb300_lastcopybytes(long long *h2d, long long *d2h) {
    *h2d = t_h2d_bytes;
    *d2h = t_d2h_bytes;
}

void cntc_gb300_resident_setup(int *n, int *ire, int *icp, int *ierror) {
    std::lock_guard<std::mutex> lk(g_res_mu);
    int rc = resident_setup(*n, ire, icp, ierror);
    if (rc != 0) {
        for (int i = 0; i < *n; i++) if (ierror[i] == 0) ierror[i] = CNTC_err_other;
        g_res.reset();
    }
}

void cntc_gb300_resident_solve(int *nrep, double *times, int *ierror) {
    std::lock_guard<std::mutex> lk(g_res_mu);
    *ierror = 0;
    if (*nrep <= 0) return;
    int rc = resident_solve(*nrep, times);
    if (rc != 0) {
        *ierror = CNTC_err_other;
        if (g_debug >= 1) std::fprintf(stderr, "contact_gb300: resident solve error %d\n", rc);
    }
}

int cntc_gb300_latencyshapes(int *cls, int *group, int *cap) { return latency_shapes(cls, group, *cap); }

int cntc_gb300_resident_graphs(void) {
    std::lock_guard<std::mutex> lk(g_res_mu);
    int c = 0;
    if (g_res) for (const ResSet &r : g_res->set) c += r.exec != nullptr;
    return c;
}

void cntc_gb300_resident_depth(int *depth) {
    std::lock_guard<std::mutex> lk(g_res_mu);
    g_res_depth = std::max(1, std::min(*depth, kMaxResidentSets));
}

void cntc_gb300_resident_collect(int *n, int *ierror) {
    std::lock_guard<std::mutex> lk(g_res_mu);
    if (!g_res || (int)g_res->b.probs.size() != *n || resident_collect(ierror) != 0)
        for (int i = 0; i < *n; i++) ierror[i] = CNTC_err_other;
}

void cntc_gb300_resident_release() {
    std::lock_guard<std::mutex> lk(g_res_mu);
    g_res.reset();
}

void cntc_gb300_getsolverstats(int *ire, int *icp, int *lenarr, double *values) {
    Problem *p = lookup(*ire, *icp, false);
    if (!p) return;
    for (int i = 0; i < *lenarr; i++) values[i] = i < (int)p->stats.size() ? p->stats[i] : 0.0;
}

} // extern "C"
