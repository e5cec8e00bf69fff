/*
 * CPU ORACLE -- test infrastructure only.
 *
 * A serial C++ restatement of CONTACT's module-3 rolling-contact solve path
 * (eve70a/CONTACT, Fortran 90), used as the parity reference of the GB300 library and
 * as the timed CPU baseline.  Nothing in the product library links or calls
 * this code; only tests/, __graft_entry__.smoke() and bench.py's CPU legs do.
 *
 * Parity pinning: the oracle reproduces the reference's golden outputs
 * testbank/test_table_mx11.ref_fx (3220 Hertzian steady-rolling cases, NormCG
 * + SteadyGS, printed to 6 decimals), the first series of
 * examples/tractcurv.ref_out (48x44 grid, 4 significant digits) and its second series (cases
 * 31-60: an elastic interfacial layer, M=4, with falling friction and a friction memory), both cases of
 * examples/cattaneo.ref_out (NormCG, TangCG on the shift problem), result
 * element 1 of testbank/test_caddon.ref_out and testbank/contact_nonhz.ref_out
 * (approach prescribed, spin) and
 * cases 1, 3, 4, 6, 7, 9-11, 13-17, 25 and 26 of testbank/testbank.ref_out (TangCG shift,
 * ConvexGS strip, SteadyGS 41x41, coupled materials, prescribed forces, transient
 * rolling from rest),
 * and the Newton-Raphson iterations on prescribed total forces of case 2 of
 * examples/cattaneo.ref_out (F=2) and case 1 of examples/catt_to_cart.ref_out
 * (F=1), the element tables of examples/carter2d.ref_out (55x1 strip,
 * SteadyGS), the five printed cases of examples/bentall.ref_out (two coupled
 * materials, chi = 180 deg, a warm-started sequence) and all 171 cases of
 * examples/catt_to_cart.ref_out (transient sequences from the previous time
 * instance), and examples/veldep_fric.ref_out (falling friction: case 1 exactly, the slip
 * iterations of the transient steps 1-34 row by row, 35-53 by count); see tests/test_oracle.py.  With the subsurface stresses it reproduces
 * all 35 load steps of examples/spence35.ref_out (tests/test_subsurf_cpu.py).  Its subsurface stresses (orc_subsurf.hpp)
 * reproduce examples/subsurf.ref_subs and the maxima of subsurf.ref_out
 * (tests/test_subsurf_cpu.py).  GDsteady (G=5) and transient rolling (T=2) have no
 * golden output in the reference: those paths are restated line by line and
 * their parity is anchored on the shared algorithms they call.
 *
 * One function solves one contact patch, the way cntc_calculate() does for one
 * (ire,icp) pair in src/contact_addon.f90:3754-3900.
 */
#ifndef CONTACT_ORACLE_H
#define CONTACT_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Inputs of one module-3 case, in CONTACT's internal units (mm, N, rad).
 * Field meanings follow t_ic / t_solvers / t_kincns in src/m_hierarch_data.f90. */
typedef struct {
    /* control digits (t_ic, m_hierarch_data.f90:134-409) */
    int pvtime, bound, tang, norm, force3, iestim, gausei;
    /* solver settings (t_solvers, m_hierarch_data.f90:739-801) */
    int maxgs, maxin, maxnr, maxout;
    double eps;
    double omegah, omegas;        /* G=2,3 */
    int    inislp;  double omgslp;
    int    kdowfb;                /* G=5 */
    double fdecay, betath, d_ifc, d_lin, d_cns, d_slp, pow_s;
    /* material, M=0 elastic (cntc_setmaterialparameters, contact_addon.f90:1287-1473) */
    double poiss1, poiss2, gg1, gg2;
    /* Coulomb friction, L=0 (contact_addon.f90:1799-1804) */
    double fstat, fkin;
    /* kinematics (t_kincns) */
    double veloc, chi, dq;
    double cksi, ceta, cphi;
    double fn, pen;
    double fxrel, fyrel;
    /* potential contact: ipotcn<0 Hertzian (params mx,my,p1,p2,scale),
     * ipotcn 1..4 explicit grid (params mx,my,p1..p4) */
    int    ipotcn;
    double potprm[6];
    /* undeformed distance (ibase 1: 6 coefficients, 9: per element) */
    int    ibase;
    int    nprmudf;
    const double *prmudf;
    /* previous solution used when iestim>0 (may be NULL) */
    const int    *igs_init;
    const double *pn_init, *px_init, *py_init;
    /* sensitivities (CNTC_ic_sens, contact_addon.f90:846): 1 none, 2 d Fn/d pen,
     * 3 also d (Fx,Fy,Mz)/d (cksi,ceta,cphi); solver limits of those solves (G=6 flags) */
    int    sens, mxsens;
    double epsens;
    /* 1: the stand-alone program's input rules (m_sinput.f90:1000-1030): MAXOUT as given for
     * dissimilar materials, where the library raises it to 10 (contact_addon.f90:1461-1462) */
    int    standalone;
    /* sensitivities of the previous case (16 values as orc_result.sens, may be NULL); kept
     * where the initial estimate keeps them (iestim 1, 3), as the creepages are */
    const double *sens_init;
    /* tractions and element division of the previous time instance for transient sequences
     * (pvtime 0: all components, 1: the normal one; may be NULL: zero, as for pvtime 2) */
    const int    *igv_init;
    const double *pvn_init, *pvx_init, *pvy_init;
    /* friction law (L digit, m_friclaw.f90): 0 Coulomb (fstat, fkin above); 2, 3, 4 falling
     * with the slip velocity, linear, rational, exponential: flaw = [fkin, f1, sabsh1, f2,
     * sabsh2] (flin / frat / fexp), with the memory distance memdst and velocity mem_s0 */
    int    frclaw;
    double flaw[5];
    double memdst, mem_s0;
    /* previous time instance of a transient sequence with falling friction: the coefficient of
     * friction and the shift per element (may be NULL) */
    const double *mus_init, *svx_init, *svy_init;
    /* material model (M digit): 0 elastic; 4 elastic bodies with an interfacial layer of modulus
     * gg3 and thickness laythk (m_sinput.f90:942-955), its flexibility laythk / gg3 added to the
     * tangential displacements; a plastic layer (tau_c0 > 0) is not restated */
    int    mater;
    double gg3, laythk, tau_c0, k_tau;
} orc_problem;

/* Outputs of one case.  Array pointers are caller-allocated with mx*my
 * entries and may be NULL. */
typedef struct {
    int ierror;                    /* as cntc_calculate: 0 ok, <0 error, >0 elements at boundary */
    int itnorm, ittang, itcg, itgs, solver;
    int mx, my;
    double dx, dy, xc1, yc1;
    double fn, fx, fy, mz, pen, elen, pmax;
    double cksi, ceta, cphi;
    double a1, b1, aa, bb, rho, cp, aob;
    int ncon, nadh, nslip;
    double *pn, *px, *py;
    double *un, *ux, *uy;
    double *sx, *sy;
    double *h;
    int    *igs;
    double *mus;                   /* coefficient of friction per element (may be NULL) */
    /* sens(iout, iin) column-major as t_output%sens: iout Fn, Fx/(mu Fn), Fy/(mu Fn), Mz;
     * iin pen, cksi, ceta, cphi (zero where not computed) */
    double sens[16];
    /* Newton-Raphson history when total forces are prescribed (F=1,2): per iteration
     * 7 values ittang, itnr, cksi, Fx/(mu Fn), ceta, Fy/(mu Fn), solver iterations; nr_hist
     * caller-allocated with room for nr_cap iterations (may be NULL), nnr = iterations made */
    int     nr_cap, nnr;
    double *nr_hist;
    /* outer iterations of the coupled normal and tangential problems (panprc): per iteration
     * the change of the tractions and its tolerance 5 eps |p| (the first 64) */
    int     nout;
    double  outer[128];
    /* iterations on the slip velocity for falling friction (L = 2..4): per iteration the
     * adhesion and slip counts, the change of the slip velocities and its tolerance
     * 0.001 |s| (the first 64) */
    int     nslp;
    double  slp[256];
} orc_result;

void orc_default_problem(orc_problem *pb);
int  orc_calculate(const orc_problem *pb, orc_result *res);

/* building blocks exposed for unit tests */
int  orc_opt_fft_size(int n);
/* influence coefficients cf(ix,iy,ik,jk), ix in [-mx,mx-1], iy in [-my,my-1];
 * out has 9*(2mx)*(2my) doubles, block (ik,jk) at offset ((ik-1)*3+(jk-1))*(4*mx*my) */
void orc_influence_coefficients(int mx, int my, double dx, double dy, double nu, double ak,
                                double xshft, double yshft, double *out);
/* u = A_ik,jk * p on a full mx*my grid via the reference's FFT convolution
 * (box = full grid); result scaled by 1/ga */
void orc_convolve(int mx, int my, const double *cf_block, double ga, const double *p, double *u);
/* same product by direct row sums (gf3_AijPj) over all elements */
void orc_convolve_direct(int mx, int my, const double *cf_block, double ga, const double *p, double *u);
/* complete elliptic integrals used by the Hertz solution */
double orc_eli(double elmodk, double *ellk, double *elle);

/* Subsurface elastic field of surface tractions pn, px, py (body 1) on an mx x my grid with
 * element centres from (xc1, yc1) and spacing dx, dy; gg, poiss [2] the two bodies (z >= 0 in
 * body 1, z < 0 in body 2).  Per point ORC_SUBS_NCOL values: ux, uy, uz, sighyd, sigvm, sigtr,
 * sigma1..3 (largest first), then the stress tensor row by row. */
#define ORC_SUBS_NCOL 18
/* at npts arbitrary points xyz[3*q..] by direct summation (m_subsurf.f90 sstres) */
void orc_subsurf_points(int mx, int my, double dx, double dy, double xc1, double yc1, const double *pn,
                        const double *px, const double *py, const double *gg, const double *poiss, int npts,
                        const double *xyz, double *out);
/* at all element centres at each of nz depths by influence coefficients and FFT convolution
 * (m_subsurf.f90 sstres_inflcf + sstres_fft); out[(iz*mx*my + ii)*ORC_SUBS_NCOL ...] */
void orc_subsurf_depths(int mx, int my, double dx, double dy, double xc1, double yc1, const double *pn,
                        const double *px, const double *py, const double *gg, const double *poiss, int nz,
                        const double *z, double *out);

#ifdef __cplusplus
}
#endif
#endif
