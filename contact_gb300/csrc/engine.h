// Host/device interface of the GB300 contact engine: one PatchDesc per contact
// patch (one cntc_calculate of one (ire,icp) pair), filled by the host API layer and
// read by the patch-solver kernel.  Plain C structs, no torch types.
#pragma once
#include <stdint.h>

namespace cgb {

// workspace columns (each npot doubles) of one patch
enum WsCol {
    W_H = 0, W_WX, W_WY,                   // undeformed distance h, rigid slip -dq*w (x,y)
    W_PX, W_PY, W_PN,                      // tractions
    W_UX, W_UY, W_UN,                      // displacement differences
    W_SX, W_SY, W_SN,                      // slip (x,y) / deformed distance (n)
    W_HSTOT, W_RHS, W_RES, W_RPRV, W_DD, W_Z, W_V, W_Q,      // NormCG
    W_WSX, W_WSY, W_DPX, W_DPY, W_DSCL, W_NX, W_NY,          // TANG
    W_RX, W_RY, W_DVX, W_DVY, W_VX, W_VY, W_QX, W_QY,
    W_POX, W_POY, W_WFX, W_WFY, W_PNX, W_PNY, W_TRC, W_ZX, W_ZY, W_ONE,   // W_WF*: fixed shift wsfix
    W_DBX, W_DBY, W_SBX, W_SBY, W_TX, W_TY,                  // mixed precision: base dp, A dp_base, change
    W_FACDT,                                                 // leading-edge fraction of the rolling step
    W_O1X, W_O1Y, W_O1N,                                     // tractions of the previous outer (NORM/TANG) iteration
    W_FLS,                                                   // 9 columns: 18 float columns of the line search
    W_FST = W_FLS + 9,                                       // 14 columns: 28 float columns of the FP32 GD state
    W_NCOL = W_FST + 14
};
enum WsIntCol { I_IGS = 0, I_OLD, I_EXT, I_IEL, I_JX, I_NCOL };

// output scalars
enum OutScalar {
    O_FN = 0, O_FX, O_FY, O_MZ, O_PEN, O_ELEN, O_PMAX,
    O_IERR, O_ITNORM, O_ITTANG, O_ITCG, O_ITGS, O_SOLVER, O_NCON, O_NADH, O_NSLIP,
    O_NCONV32, O_NCONV64, O_NLS, O_STATUS,
    O_T_TOTAL, O_T_CONV, O_T_LS, O_T_DIAG, O_T_GS, O_T_NORM, O_T_TANG, O_T_SCAN,   // SM clock cycles
    O_T_CONV32,                            // SM cycles in FP32 convolutions (part of O_T_CONV)
    O_T_GSSER,                             // SM cycles of the serial element steps of SteadyGS (part of O_T_GS)
    O_ALGB,                                // algorithmic bytes of the convolutions (inputs, spectra, outputs)
    O_TSTART, O_TEND,                      // global timer (ns) at the start and end of the solve
    O_CKSI, O_CETA,                        // creepages (solved for when total forces are prescribed)
    O_SENS,                                // 16: d(Fn, Fx, Fy, Mz) / d(pen, cksi, ceta, cphi), [out * 4 + in]
    O_NSCAL = O_SENS + 16
};

// solver status bits (O_STATUS)
constexpr int ST_OK = 0, ST_UNSUPPORTED = 1, ST_NOBRACKET = 2, ST_NORMCG_DIV = 4, ST_BADSIZE = 8, ST_GROUPFAIL = 16;

struct PatchDesc {
    int mx, my, npot;
    int fx, fy;                       // FFT grid NX = 2 fx, NY = 2 fy
    double dx, dy, dxdy, xc1, yc1;
    int tang, norm, bound, iestim, force3, gausei;
    int maxgs, maxin, maxout;
    double eps;
    double omegah, omegas;
    int gd_meth, kdown, kdowfb;
    double fdecay, betath, d_ifc, d_lin, d_cns, d_slp, pow_s;
    double ga, nu, ak;                // combined modulus, Poisson ratio and difference parameter K
    double fstat;
    double chi, dq, cksi, ceta, cphi;
    double fntrue, pen;
    int ihertz;
    double aa, bb;
    int ibase;
    double prm[6];
    int precision;                    // 0: FP64 throughout; 1-3: mixed-precision tiers (see gdsteady)
    double eps32;                     // tolerance of the FP32 phase
    int maxnr;                        // Newton-Raphson iterations on prescribed total forces
    double fxrel, fyrel;              // prescribed Fx / (mu Fn), Fy / (mu Fn) (force3 >= 1, >= 2)
    double sens0[16];                 // sensitivities of the previous solve (warm start), [out * 4 + in]
    int sens;                         // S digit: >= 2 d Fn / d pen, >= 3 also the creepage sensitivities
    int mxsens;                       // iterations and tolerance of the sensitivity solves
    double epsens;
    int pvtime;                       // P digit: 0 previous time instance, 1 its normal part, 2 none
    int ncf;                          // coefficient blocks in cf: 4 (K = 0), 6 (K != 0), 8 (K != 0, steady rolling)
    // previous solution of the problem in device memory (prev_block layout), or nullptr: the
    // initial estimate when iestim != 0 and the previous time instance when pvtime <= 1.
    // save: where the solve leaves its own solution in the same layout (may equal prev), or nullptr.
    const double *prev;
    double *save;
    // completion flag of the patch in host-mapped memory (serving), or nullptr: set to 1 after
    // all results of the patch are in its io block and fenced at system scope
    int *done;
    // io block: columns W_H .. W_SN (kIoCols * npot doubles), then O_NSCAL output scalars,
    // then the element division (npot ints).  Inputs (element-wise h, warm-start tractions
    // and element division) arrive and all results leave through this block.
    double *io;
    double *wk;                       // work columns W_HSTOT .. (W_NCOL - kIoCols) * npot doubles
    int *wki;                         // int columns I_OLD .. ((I_NCOL - 1) * npot ints)
    // spatial influence coefficients [ncf][2my][2mx]: xx, xy, yy, zz; with K != 0 also xz, yz
    // (zx = -xz, zy = -yz) and, in steady rolling, xz and yz of cs - cv (cv: the grid shifted by
    // one rolling step)
    const double *cf;
    // spectra [spectra_count(ncf)][fx+1][fy+1]: xx, xy, yy, zz, M_zz, M_xx, M_yy; with K != 0 the
    // imaginary parts of xz, yz, and in steady rolling the real and imaginary parts of xz and of
    // yz of cs - cv
    const double *spec64;
    const float *spec32;
    void *rbuf;                       // 2 * (fx+1) * my complex doubles
    // patch group: nblk CTAs solve the patch together (1: a single CTA); gscr holds their
    // barrier, reduction partials and twiddle tables (nblk > 1 only)
    int nblk;
    int pad2_;
    void *gscr;
};

constexpr int kNumPhaseTimers = 10;  // O_T_TOTAL .. O_T_GSSER
constexpr int kIoCols = W_HSTOT;      // W_H .. W_SN live in the io block

// SteadyGS and ConvexGS visit the elements one after another: a patch group refuses them above
// this many elements (a sweep would take seconds)
constexpr int kMaxGroupGsElements = 40000;

// spectra of a patch with ncf coefficient blocks (PatchDesc::spec64)
__host__ __device__ inline int spectra_count(int ncf) { return ncf >= 8 ? 13 : (ncf >= 6 ? 9 : 7); }

__host__ __device__ inline size_t io_doubles(int npot) {
    return (size_t)kIoCols * npot + O_NSCAL + (size_t)(npot + 1) / 2;
}

// block of a problem's previous solution: px, py, pn (npot doubles each), then the element
// division (npot ints)
__host__ __device__ inline size_t prev_bytes(int npot) {
    return ((size_t)3 * npot * sizeof(double) + (size_t)npot * sizeof(int) + 255) & ~(size_t)255;
}

} // namespace cgb
