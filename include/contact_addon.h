/*
 * contact_addon.h -- C-ABI of the GB300 rolling-contact library.
 *
 * A drop-in for the module-3 part of CONTACT's library interface: same lowercase
 * symbol names, same argument lists (every argument by pointer, Fortran bind(c)
 * convention), same argument meaning and units.  The reference prototypes are in
 * matlab_intfc/contact_addon.h; the Fortran implementations are cited per function
 * below (file:line in src/contact_addon.f90 unless stated otherwise).
 *
 * Additions (no counterpart in the reference):
 *   cntc_calculate_batch        solve many (ire,icp) problems in one pass of the engine
 *   cntc_getiterationcounts     iteration counts / solver used of the last solve
 *   cntc_gb300_kernel_launches  number of GPU kernels this library has launched
 *   cntc_gb300_getsolverstats   convolution counts and per-phase cycle counts of the last solve
 *   cntc_gb300_resident_*       solve a staged batch repeatedly on device-resident inputs
 *   cntc_gb300_fmapeaks         measured FP64 / FP32 FMA peaks of the device
 *   cntc_gb300_latencyshapes    launch shapes tuned per size class for single-patch calls
 *   flag CNTC_if_mixedprec      (cntc_setflags) 1: FP32 convolutions + FP64 refinement
 *   flag CNTC_if_groupctas      (cntc_setflags) CTAs per patch: one, or a cooperative group
 */
#ifndef CONTACT_GB300_ADDON_H
#define CONTACT_GB300_ADDON_H

#ifdef __cplusplus
extern "C" {
#endif

/* library extension flag for cntc_setflags: 0 = FP64 throughout (default); mixed precision,
 * the FP64 iteration path with FP64 residual replacement: 1 = FP32 convolution products,
 * 2 = also FP32 diagonal scaling and local element solves, 3 = also an FP32 line search,
 * 4 = GDsteady on an FP32 state until single precision stops resolving the change, then the
 * same iteration continued on the FP64 state with tier-2 arithmetic */
#define CNTC_if_mixedprec 2010

/* library extension flag for cntc_setflags: CTAs that solve one patch together.  0 (default):
 * one CTA per patch when the grid's FFT lines fit the per-warp shared-memory buffers (grid
 * sides up to about 210), else a cooperative group of up to one CTA per 256 elements, bounded
 * by the CTAs the device holds at once; 1: one CTA only (larger grids return CNTC_err_other);
 * n >= 2: a group of at most n CTAs for any grid */
#define CNTC_if_groupctas 2011

/* initialisation: cntc_initializeFirst 235-442, cntc_initializeFirst_new 446-472,
 * cntc_initialize 476-576 */
void cntc_initializefirst(int *ifcver, int *ierror, int *ioutput, const char *c_wrkdir,
                          const char *c_outdir, const char *c_expnam, int *len_wrkdir,
                          int *len_outdir, int *len_expnam);
void cntc_initializefirst_new(int *ifcver, int *ierror, int *ioutput, const char *c_wrkdir,
                              const char *c_outdir, const char *c_expnam, int *len_wrkdir,
                              int *len_outdir, int *len_expnam);
void cntc_initialize(int *ire, int *imodul, int *ifcver, int *ierror, const char *c_outdir,
                     int *len_outdir);

/* configuration: cntc_setGlobalFlags 580-725, cntc_setFlags 780-973,
 * cntc_setSolverFlags 1128-1283, cntc_setMaterialParameters 1287-1473,
 * cntc_setTemperatureData 1477-1550, cntc_setTimestep 1554-1583,
 * cntc_setReferenceVelocity 1587-1615, cntc_setRollingStepsize 1619-1667,
 * cntc_setFrictionMethod 1671-1968 */
void cntc_setglobalflags(int *lenflg, int *params, int *values);
void cntc_setflags(int *ire, int *icp, int *lenflg, int *params, int *values);
void cntc_setsolverflags(int *ire, int *icp, int *gdigit, int *nints, int *iparam, int *nreals,
                         double *rparam);
void cntc_setmaterialparameters(int *ire, int *icp, int *mdigit, int *nparam, double *rparam);
void cntc_settemperaturedata(int *ire, int *icp, int *imeth, int *nparam, double *rparam);
void cntc_settimestep(int *ire, int *icp, double *dt);
void cntc_setreferencevelocity(int *ire, int *icp, double *veloc);
void cntc_setrollingstepsize(int *ire, int *icp, double *chi, double *dq);
void cntc_setfrictionmethod(int *ire, int *icp, int *imeth, int *nparam, double *params);

/* geometry and loading: cntc_setHertzContact 1972-2093, cntc_setPotContact 2097-2257,
 * cntc_setPenetration 2294-2323, cntc_setNormalForce 2327-2357,
 * cntc_setUndeformedDistc 2361-2487, cntc_setCreepages 2491-2530,
 * cntc_setExtraRigidSlip 2534-2593, cntc_setTangentialForces 2597-2650 */
void cntc_sethertzcontact(int *ire, int *icp, int *ipotcn, int *nparam, double *rparam);
void cntc_setpotcontact(int *ire, int *icp, int *ipotcn, int *nparam, double *rparam);
void cntc_setpenetration(int *ire, int *icp, double *pen);
void cntc_setnormalforce(int *ire, int *icp, double *fn);
void cntc_setundeformeddistc(int *ire, int *icp, int *ibase, int *nparam, double *prmudf);
void cntc_setcreepages(int *ire, int *icp, double *vx, double *vy, double *phi);
void cntc_setextrarigidslip(int *ire, int *icp, int *lenarr, double *wx, double *wy);
void cntc_settangentialforces(int *ire, int *icp, double *fx, double *fy);

/* computation: cntc_calculate 3519-3552 -> cntc_calculate3 3754-3900 */
void cntc_calculate(int *ire, int *icp, int *ierror);
/* extension: n problems (ire[i], icp[i]) solved together; ierror[i] as cntc_calculate */
void cntc_calculate_batch(int *n, int *ire, int *icp, int *ierror);
/* extension, no counterpart in the reference: cntc_calculate that allocates no device memory.
 * All device buffers of the solve come from a fixed 16 MiB device array of the library
 * (grids up to about 140 x 140; larger problems return CNTC_err_other with a message).  The
 * one array serves every call of the process, so overlapping calls would race on it; the
 * library serialises them with a lock and each call waits for its own work to finish
 * before it returns.  The first call of a process looks up the array's device address and
 * creates the library's streams: make it before any stream capture of the caller. */
void cntc_calculate_noalloc(int *ire, int *icp, int *ierror);
/* extension (serving): queue the solve of (ire, icp) and return at once (ierror 0 when
 * queued).  Queued solves are batched by free worker lanes as they arrive, up to a device
 * memory admission budget, and run concurrently with earlier batches.  The problem's
 * settings must not change until cntc_wait has returned for it; a second request for the
 * same problem before then is refused with CNTC_err_other. */
void cntc_calculate_async(int *ire, int *icp, int *ierror);
/* extension (serving): wait for a queued solve; ierror as cntc_calculate */
void cntc_wait(int *ire, int *icp, int *ierror);
/* extension: cntc_wait that also returns the time from queueing to completion (seconds) */
void cntc_gb300_wait_latency(int *ire, int *icp, int *ierror, double *latency);
/* extension: device-memory admission budget of the serving queue in GB (default 40) */
void cntc_gb300_setadmissionbudget(double *gbytes);

/* results: cntc_getFlags 4001-4160, cntc_getReferenceVelocity 4987-5017,
 * cntc_getHertzContact 5021-5066, cntc_getNumElements 5070-5099,
 * cntc_getGridDiscretization 5103-5140, cntc_getPotContact 5144-5187,
 * cntc_getPenetration 5191-5220, cntc_getCreepages 5224-5271,
 * cntc_getContactForces 5275-5318, cntc_getContactPatchAreas 5460-5497,
 * cntc_getElementDivision 5501-5552, cntc_getMaximumPressure 5556-5587,
 * cntc_getMaximumTraction 5591-5626, cntc_getFieldData 5672-5823,
 * cntc_getTractions 5827-5855, cntc_getMicroSlip 5859-5885,
 * cntc_getDisplacements 5889-5915, cntc_getSensitivities 5919-6007,
 * cntc_getCalculationTime 6011-6040, cntc_resetCalculationTime 6044-6067 */
void cntc_getflags(int *ire, int *icp, int *lenflg, int *params, int *values);
void cntc_getreferencevelocity(int *ire, int *icp, double *veloc);
void cntc_gethertzcontact(int *ire, int *icp, int *lenarr, double *values);
void cntc_getnumelements(int *ire, int *icp, int *mx, int *my);
void cntc_getgriddiscretization(int *ire, int *icp, double *dx, double *dy);
void cntc_getpotcontact(int *ire, int *icp, int *lenarr, double *values);
void cntc_getpenetration(int *ire, int *icp, double *pen);
void cntc_getcreepages(int *ire, int *icp, double *vx, double *vy, double *phi);
void cntc_getcontactforces(int *ire, int *icp, double *fn, double *tx, double *ty, double *mz);
void cntc_getcontactpatchareas(int *ire, int *icp, double *carea, double *harea, double *sarea);
void cntc_getelementdivision(int *ire, int *icp, int *lenarr, int *eldiv);
void cntc_getmaximumpressure(int *ire, int *icp, double *pnmax);
void cntc_getmaximumtraction(int *ire, int *icp, double *ptmax);
void cntc_getfielddata(int *ire, int *icp, int *ifld, int *lenarr, double *fld);
void cntc_gettractions(int *ire, int *icp, int *lenarr, double *pn, double *px, double *py);
void cntc_getmicroslip(int *ire, int *icp, int *lenarr, double *sx, double *sy);
void cntc_getdisplacements(int *ire, int *icp, int *lenarr, double *un, double *ux, double *uy);
void cntc_getsensitivities(int *ire, int *icp, int *lenout, int *lenin, double *sens);
void cntc_getcalculationtime(int *ire, int *icp, double *tcpu, double *twall);
void cntc_resetcalculationtime(int *ire, int *icp);
/* extension: [itnorm, ittang, itcg, itgs, solver id, ierror] of the last solve */
void cntc_getiterationcounts(int *ire, int *icp, int *lenarr, int *values);

/* module 3 parameters: cntc_getParameters 4164-4258 (itask 1 kinematics, 2 material,
 * 3 friction; values in the selected units) */
void cntc_getparameters(int *ire, int *icp, int *itask, int *lenarr, double *values);
/* metadata for output files only: cntc_setMetadata 1055-1124 (accepted, no effect on a solve) */
void cntc_setmetadata(int *ire, int *icp, int *lenmta, int *params, double *values);
/* temperature (not computed here, heat digit 0): cntc_getMaximumTemperature 5630-5668;
 * returns 0, 0 as the reference does without a temperature solution */
void cntc_getmaximumtemperature(int *ire, int *icp, double *t1max, double *t2max);

/* Entry points of the wheel-rail module (module 1) and the input-file reader.  They lie
 * outside this library's solve path; they are exported so that hosts binding the reference's
 * full interface load this library unchanged.  Each logs that it is not supported and returns:
 * setters without effect, getters with zero outputs, and ierror = CNTC_err_other where the
 * call has one.  The subsurface entry points (subs_*) below them are implemented for module 3
 * (see their own comment).  Fortran implementations:
 * cntc_readInpFile 729-776, cntc_setVerticalForce 2261-2290, cntc_setProfileInputFname
 * 2654-2749, cntc_setProfileInputValues 2753-2829, cntc_setTrackDimensions 2833-2985,
 * cntc_setWheelsetDimensions 2989-3063, cntc_setWheelsetPosition 3067-3132,
 * cntc_setWheelsetVelocity 3136-3214, cntc_setWheelsetFlexibility 3218-3326,
 * cntc_getProfileValues 4262-4693, cntc_getProfileValues_new 4697-4718,
 * cntc_getWheelsetPosition 4722-4752, cntc_getWheelsetVelocity 4756-4786,
 * cntc_getNumContactPatches 4790-4812, cntc_getContactLocation 4816-4983,
 * cntc_getGlobalForces 5322-5456, subs_addBlock 3330-3515, subs_calculate 3904-3997,
 * subs_getBlocksize 6071-6109, subs_getResults 6113-6187 */
void cntc_readinpfile(int *ire, int *inp_type, const char *c_fname, int *len_fname, int *ierror);
void cntc_setverticalforce(int *ire, double *fz);
void cntc_setprofileinputfname(int *ire, const char *c_fname, int *len_fname, int *nints, int *iparam,
                               int *nreals, double *rparam);
void cntc_setprofileinputvalues(int *ire, int *npoint, double *values, int *nints, int *iparam, int *nreals,
                                double *rparam);
void cntc_settrackdimensions(int *ire, int *ztrack, int *nparam, double *rparam);
void cntc_setwheelsetdimensions(int *ire, int *ewheel, int *nparam, double *rparam);
void cntc_setwheelsetposition(int *ire, int *ewheel, int *nparam, double *rparam);
void cntc_setwheelsetvelocity(int *ire, int *ewheel, int *nparam, double *rparam);
void cntc_setwheelsetflexibility(int *ire, int *ewheel, int *nparam, double *rparam);
void cntc_getprofilevalues(int *ire, int *itask, int *nints, int *iparam, int *nreals, double *rparam, int *lenarr,
                           double *values);
void cntc_getprofilevalues_new(int *ire, int *itask, int *nints, int *iparam, int *nreals, double *rparam,
                               int *lenarr, double *values);
void cntc_getwheelsetposition(int *ire, int *lenarr, double *values);
void cntc_getwheelsetvelocity(int *ire, int *lenarr, double *values);
void cntc_getnumcontactpatches(int *ire, int *npatch);
void cntc_getcontactlocation(int *ire, int *icp, int *lenarr, double *values);
void cntc_getglobalforces(int *ire, int *icp, int *lenarr, double *values);
/* Subsurface stresses of module 3 (src/contact_addon.f90 subs_addBlock 3330-3515,
 * subs_calculate 3904-3997, subs_getBlocksize 6071-6109, subs_getResults 6113-6187;
 * m_subsurf.f90): blocks of points (types 1-3, 5-7: element centres selected by index ranges or
 * lists at regular or listed depths; 9: x, y, z lists), evaluated on the GPU for the tractions
 * of the problem's last solve (z >= 0 in body 1, z < 0 in body 2).  Results per point: x, y, z,
 * displacements, hydrostatic / von Mises / Tresca stress, principal stresses and the stress
 * tensor by columns (21 columns, points x fastest, then y, then z).  subs_calculate on a
 * problem without a solution returns CNTC_err_other. */
void subs_addblock(int *ire, int *icp, int *iblk, int *isubs, int *nx, int *ny, int *nz, double *xparam,
                   double *yparam, double *zparam);
void subs_calculate(int *ire, int *icp, int *ierror);
void subs_getblocksize(int *ire, int *icp, int *iblk, int *nx, int *ny, int *nz);
void subs_getresults(int *ire, int *icp, int *iblk, int *lenarr, int *ncol, int *icol, double *values);

/* clean-up: cntc_finalize 6243-6290, cntc_finalizeLast 6294-6375 */
void cntc_finalize(int *ire);
void cntc_finalizelast(void);

/* extension: number of GPU kernels launched by this library since it was loaded */
long long cntc_gb300_kernel_launches(void);
/* extension: engine statistics of the last solve of (ire,icp): [0] FP32 convolutions,
 * [1] FP64 convolutions, [2] line-search steps, [3] status bits, [4..12] SM clock cycles
 * spent in: whole solve, convolutions, line search, diagonal scaling, Gauss-Seidel sweeps,
 * normal problem, tangential problem, row scans, FP32 convolutions; [13] algorithmic bytes
 * of the convolutions; [14], [15] GPU global timer (ns) at the start and end of the solve;
 * [16] CTAs that solved the patch */
void cntc_gb300_getsolverstats(int *ire, int *icp, int *lenarr, double *values);

/* extension (no reference counterpart): resident batch for throughput measurement.
 * setup prepares the n problems (ire[i], icp[i]) and stages their inputs in device memory
 * (ierror[i] as cntc_calculate for problems that cannot be prepared); solve runs the whole
 * engine nrep times on the staged inputs, influence coefficients included, and writes per
 * run 4 values: device ms of the pass, ms in patch-solve kernels, ms in influence/spectrum
 * kernels (CUDA events on the launching stream) and the number of launches; collect copies
 * the results of the last run back to the problems (getters then work as after
 * cntc_calculate); release frees the device memory. */
void cntc_gb300_resident_setup(int *n, int *ire, int *icp, int *ierror);
/* extension: bytes copied host->device and device->host by the calling thread's last
 * cntc_calculate / cntc_calculate_batch */
void cntc_gb300_lastcopybytes(long long *h2d, long long *d2h);
void cntc_gb300_resident_solve(int *nrep, double *times, int *ierror);
void cntc_gb300_resident_collect(int *n, int *ierror);
void cntc_gb300_resident_release(void);
/* extension (no reference counterpart): number of buffer sets (1..4, default 1) of the next
 * cntc_gb300_resident_setup.  With depth d > 1 consecutive passes of cntc_gb300_resident_solve
 * overlap: pass r runs in set r mod d on its own streams, so the SMs that the last patches of a
 * pass leave idle take the next passes' patches (continuous batching).  times[4r] is then the
 * device time of all nrep passes divided by nrep. */
void cntc_gb300_resident_depth(int *depth);
/* extension (no reference counterpart): number of buffer sets of the resident batch whose pass
 * is replayed from a captured CUDA graph (influence coefficients, spectra and the persistent
 * solve launch); sets with patch groups launch directly. */
int cntc_gb300_resident_graphs(void);
/* extension (no reference counterpart): FMA peaks of the current device, measured with CUDA
 * events: out[0] FP64, out[1] FP32, in TFLOP/s.  The denominators of the patch-solve kernel's
 * arithmetic roofline.  Returns 0, or -1 when a measurement failed. */
int cntc_gb300_fmapeaks(double *out);
/* extension (no reference counterpart): launch shapes chosen so far for single-patch calls
 * (cntc_calculate): per entry the size class c (grids of 2^c .. 2^(c+1) - 1 elements) and
 * whether a cooperative group of CTAs (1) or one CTA (0) solves it, as timed on the device the
 * first time the class was met.  Returns the number of entries written (at most *cap). */
int cntc_gb300_latencyshapes(int *cls, int *group, int *cap);

#ifdef __cplusplus
}
#endif
#endif
