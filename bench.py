"""Throughput benchmark of the GB300 rolling-contact library on the batched mixed-size workload.

Workload: 4096 independent Hertzian steady-rolling patches (seed 2): grid sides U{24..160},
semi-axes log-uniform 2-10 mm, Fn U[10,150] kN, creepages U[-0.005,0.005], spin U[-0.5,0.5]
rad/m, mu U[0.2,0.4], steel on steel; NormCG + GDsteady with FP32 convolutions and FP64
refinement to eps 1e-8.  One step = one solve of all patches (influence coefficients,
normal and tangential problem, force integration).

  value  solves/s with inputs resident in device memory (cntc_gb300_resident_*; CUDA events
         on the library's stream around its launches)
  e2e    solves/s through cntc_calculate_batch from host buffers (host->device copy of the
         inputs, device->host copy of all results inside the timed region)
  --impl reference  the CPU oracle (serial restatement of the reference's solve path) on
         all host cores, on a bounded sample of the same workload per step

Multi-GPU: patches are independent and nothing is exchanged, so N ranks run N replicas of
the workload (weak scaling); value = total solves / max over ranks of the timed region.
"""
import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (ROOT, os.path.join(ROOT, "tests")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import cases as C  # noqa: E402

T_START = time.perf_counter()
METRIC = "solves/s & p99 latency, mixed+batched vs plain FP64 on GB300 at 1e-8 rel err"
UNIT = "solves/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--patches", type=int, default=4096)
    ap.add_argument("--seed", type=int, default=2)
    ap.add_argument("--plain-sample", type=int, default=608,
                    help="patches of the same workload solved in plain FP64 for the mixed/plain ratio")
    ap.add_argument("--depth", type=int, default=3,
                    help="buffer sets of the resident batch: consecutive passes overlap over this many sets "
                         "(continuous batching across steps); 1 runs the passes one after another")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-threads", type=int, default=0, help="host threads of the CPU legs (0: all)")
    ap.add_argument("--cpu-max-side", type=int, default=0,
                    help="test aid: draw the CPU sample from patches with both sides <= this (0: all sizes)")
    ap.add_argument("--time-budget", type=float, default=1500.0,
                    help="wall-clock seconds the default run must end within; timed passes that would not fit "
                         "are not run (the line reports steps run and steps requested)")
    ap.add_argument("--max-side", type=int, default=0,
                    help="profiling aid: keep only patches with both sides <= this (0: all)")
    ap.add_argument("--serving", action="store_true",
                    help="serving stream (wheels x 2 patches, random-walk loads, Poisson arrivals, warm start)")
    ap.add_argument("--wheels", type=int, default=256)
    ap.add_argument("--time-steps", type=int, default=3)
    ap.add_argument("--rate", type=float, default=25.0, help="Poisson arrival rate, requests/s")
    ap.add_argument("--large", action="store_true",
                    help="large single patch: 1024^2 rough surface (Fn 150 kN, creepages 0.003/0/0.3 rad/m, "
                         "mu 0.25), FP64 against FP32 convolutions + FP64 refinement, solved by a CTA group")
    ap.add_argument("--perfc", action="store_true",
                    help="the reference's own performance inputs (perfc_test: normal problems 71x81 to 575x647, "
                         "shift problems), FP64, each through cntc_calculate, against the published 2016 timings")
    ap.add_argument("--accuracy", action="store_true",
                    help="errors of the mixed and FP64 forms at the workload's eps and at --tight-eps, each against "
                         "the others, on the first --plain-sample patches")
    ap.add_argument("--tight-eps", type=float, default=1e-11)
    ap.add_argument("--large-side", type=int, default=1024)
    ap.add_argument("--large-maxgs", type=int, default=3000)
    ap.add_argument("--large-eps", type=float, default=1e-6,
                    help="GDsteady tolerance of the large patch (at 1e-8 GDsteady needs more than 5000 iterations "
                         "at 1024^2)")
    return ap.parse_args()


MIXED_TIER = 1     # FP32 convolution products along the FP64 iteration path
# DRAM bytes (read + write) per algorithmic byte of k_solve, from one ncu capture of the
# persistent solve on 304 patches with sides <= 64, two CTAs per SM: 41.5 GB of DRAM traffic
# against 71.4 GB of algorithmic bytes in the same launch (the bench's own count).  The full
# workload is too large to capture; its traffic is estimated with this ratio.
TRAFFIC_PER_ALG_BYTE = 41.5 / 71.4


def workload(n, seed, mixed=MIXED_TIER, max_side=0):
    if max_side <= 0:
        return C.batch_patches(n, seed=seed, mixed=mixed, eps=1e-8)
    allc = C.batch_patches(4096, seed=seed, mixed=mixed, eps=1e-8)
    return [c for c in allc if c["potprm"][0] <= max_side and c["potprm"][1] <= max_side][:n]


# ------------------------------------------------------------------------------------------
# distributed plumbing (torchrun): replicas, barrier, max over ranks
# ------------------------------------------------------------------------------------------
class Dist:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist
            backend = "nccl" if _cuda_ok() else "gloo"
            dist.init_process_group(backend=backend)
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, v):
        if not self.pg:
            return v
        import torch
        dev = "cuda" if _cuda_ok() else "cpu"
        t = torch.tensor([float(v)], dtype=torch.float64, device=dev)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def sum(self, v):
        if not self.pg:
            return v
        import torch
        dev = "cuda" if _cuda_ok() else "cpu"
        t = torch.tensor([float(v)], dtype=torch.float64, device=dev)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


def _cuda_ok():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


# ------------------------------------------------------------------------------------------
# clocks sampled during the timed region
# ------------------------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []
        self.t = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.t:
            self.t.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for ln in self.lines:
            v = [x.strip() for x in ln.split(",")]
            if len(v) < 9:
                continue
            try:
                sm.append(float(v[1]))
                smax.append(float(v[2]))
            except ValueError:
                continue
            for name, flag in zip(names, v[5:9]):
                if flag.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# ------------------------------------------------------------------------------------------
# CPU baseline: the oracle on all host cores, on a sample stratified over the workload's sizes
# ------------------------------------------------------------------------------------------
def stratified_sample(cases, nstrata, seed):
    """One patch from each of nstrata equal-count strata of the workload ordered by element
    count, drawn with the given seed: every stratum weighs 1/nstrata of the workload, so the
    mean time over the sample estimates the workload's mean time per patch."""
    rng = np.random.default_rng(seed)
    order = sorted(range(len(cases)), key=lambda i: (cases[i]["potprm"][0] * cases[i]["potprm"][1], i))
    edges = np.linspace(0, len(order), nstrata + 1).astype(int)
    return [order[int(rng.integers(edges[k], edges[k + 1]))] for k in range(nstrata) if edges[k + 1] > edges[k]]


def cpu_sample_rate(cases, seed, threads=None, nstrata=None):
    """Solve a stratified sample of the workload (one patch per size stratum, sides 24-160
    alike) with the CPU oracle's baseline build (Stockham FFT, real-input convolutions) on a
    thread pool, one patch per thread at a time as the reference's OpenMP patch loop does
    (ctypes releases the GIL).  Throughput = threads x patches / (sum of per-patch seconds):
    the rate of a pool that stays busy on the whole workload, measured on patches of every
    size with no extrapolation.  Returns (solves/s, threads, description, wall seconds)."""
    from concurrent.futures import ThreadPoolExecutor
    import pyoracle as po
    po.build()
    threads = threads or os.cpu_count() or 1
    nstrata = nstrata or threads
    idx = stratified_sample(cases, nstrata, seed)

    def one(i):
        c = dict(cases[i], mixed=0)
        ts = time.perf_counter()
        C.oracle_solve(c, fast=True)
        return time.perf_counter() - ts

    t0 = time.perf_counter()
    with ThreadPoolExecutor(max_workers=threads) as ex:
        times = list(ex.map(one, idx))
    wall = time.perf_counter() - t0
    rate = threads * len(idx) / sum(times)
    sides = sorted(int(cases[i]["potprm"][0]) * int(cases[i]["potprm"][1]) for i in idx)
    desc = ("%d patches of the workload, one per equal-count stratum of element count (%d to %d elements, "
            "sides 24-160: stratified over the full range, no extrapolation), solved by the oracle's baseline "
            "build on %d threads in %.1f s wall; rate = threads x patches / sum of per-patch seconds"
            % (len(idx), sides[0], sides[-1], threads, wall))
    return rate, threads, desc, wall


def small_patch_latency(cg, reps=5):
    """One small patch in a single call: the 21 x 21 Hertzian steady-rolling case of the smoke
    test (GDsteady, FP64, eps 1e-10) through cntc_calculate (wall time, host buffers, median of
    reps calls on a fresh problem each, after one warm-up call), beside the oracle's baseline
    build on one core."""
    import torch
    case = C.config0(gausei=5, eps=1e-10, mx=21, my=21)
    gpu = []
    for r in range(reps + 1):
        cg.setup_case(900 + r, 1, case)
        torch.cuda.synchronize()
        t = time.perf_counter()
        cg.calculate(900 + r, 1)
        torch.cuda.synchronize()
        if r > 0:
            gpu.append(time.perf_counter() - t)
        st, it = cg.getsolverstats(900 + r, 1), cg.getiterationcounts(900 + r, 1)
        cg.finalize(900 + r)
    tot = max(st["t_total"], 1.0)
    phases = {k[2:]: round(st[k] / tot, 3) for k in ("t_norm", "t_tang", "t_conv", "t_ls", "t_scan", "t_diag")}
    import pyoracle as po
    po.build()
    cpu = []
    for r in range(reps):
        t = time.perf_counter()
        C.oracle_solve(case, fast=True)
        cpu.append(time.perf_counter() - t)
    return {"case": "21 x 21 Hertzian steady rolling, GDsteady, FP64, eps 1e-10, one cntc_calculate",
            "gpu_ms": float(np.median(gpu) * 1e3), "cpu_one_core_ms": float(np.median(cpu) * 1e3),
            "kernel_ms": st["t_total"] / 2.07e6, "gd_iterations": it["itgs"], "nconv64": st["nconv64"],
            "phase_share_of_sm_cycles": phases,
            "note": "single-call latency of one small patch (one CTA); the CPU is the oracle's baseline build"}


# ------------------------------------------------------------------------------------------
# GB300 arm
# ------------------------------------------------------------------------------------------
def _fields(cg, ire, icp):
    fn, fx, fy, _ = cg.getcontactforces(ire, icp)
    pn, px, py = cg.gettractions(ire, icp)
    return dict(fn=fn, fx=fx, fy=fy, pmax=cg.getmaximumpressure(ire, icp), pn=pn, px=px, py=py,
                igs=np.asarray(cg.getelementdivision(ire, icp)).ravel())


def form_errors(cg, ire, icp_a, icp_b, fstat):
    """Per patch, form a (icp_a) against form b (icp_b) of the same problems: tangential force
    |dF_t| / max(|F_t|, 1e-3 mu Fn), normal force |dFn| / Fn, maximum pressure |dpmax| / pmax,
    traction field max |dp| / pmax over the three components, and the elements whose class
    differs."""
    out = {k: [] for k in ("ft", "fn", "pmax", "tractions", "eldiv")}
    for i, mu in zip(ire, fstat):
        a, b = _fields(cg, i, icp_a), _fields(cg, i, icp_b)
        ft = math.hypot(b["fx"], b["fy"])
        out["ft"].append(math.hypot(a["fx"] - b["fx"], a["fy"] - b["fy"]) / max(ft, 1e-3 * mu * abs(b["fn"])))
        out["fn"].append(abs(a["fn"] - b["fn"]) / max(abs(b["fn"]), 1e-300))
        out["pmax"].append(abs(a["pmax"] - b["pmax"]) / max(b["pmax"], 1e-300))
        dp = max(float(np.abs(a[k] - b[k]).max()) for k in ("pn", "px", "py"))
        out["tractions"].append(dp / max(b["pmax"], 1e-300))
        out["eldiv"].append(int((a["igs"] != b["igs"]).sum()))
    return {k: np.array(v) for k, v in out.items()}


def summarize_errors(errs, bound=1e-8):
    out = {}
    for k, v in errs.items():
        if k == "eldiv":
            out[k] = {"patches_differing": int((v > 0).sum()), "max_elements": int(v.max())}
        else:
            out[k] = {"median": float(np.median(v)), "p99": float(np.percentile(v, 99)), "max": float(v.max()),
                      "above_%g" % bound: int((v > bound).sum())}
    return out


def setup_problems(cg, cases, ire0=1):
    ire = list(range(ire0, ire0 + len(cases)))
    for i, c in zip(ire, cases):
        cg.setup_case(i, 1, c)
    return ire, [1] * len(cases)


def run_gb300(args, dist):
    import torch
    import contact_gb300 as cg
    torch.cuda.set_device(dist.local)
    cg.load()
    cases = workload(args.patches, args.seed, mixed=MIXED_TIER, max_side=args.max_side)
    n = len(cases)
    ire, icp = setup_problems(cg, cases)
    rb = cg.ResidentBatch(ire, icp, depth=args.depth)
    bad = int((rb.setup_errors != 0).sum())
    if bad:
        raise RuntimeError("%d patches could not be prepared" % bad)
    # warm-up passes, one at a time; the wall time of the last one sizes the rest of the run
    t_pass = 0.0
    for _ in range(args.warmup):
        tw = time.perf_counter()
        rb.solve(1)
        t_pass = time.perf_counter() - tw
    # wall-clock guard: the timed passes, the plain-FP64 sample (about 0.4 of a pass with its
    # mixed twin), the end-to-end pass and the CPU leg must end within --time-budget seconds
    # of the start; fewer timed passes are run (and reported) only if they would not
    reserve = 1.6 * t_pass + 90.0
    avail = args.time_budget - (time.perf_counter() - T_START) - reserve
    steps = args.steps
    if t_pass > 0 and avail < steps * t_pass:
        steps = max(1, int(avail // t_pass))
    steps = int(-dist.max(-steps))          # the smallest count over the ranks
    dist.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(dist.local)
    clocks.start()
    launches1 = cg.kernel_launches()
    times = rb.solve(steps)
    gpu_launches = cg.kernel_launches() - launches1
    torch.cuda.synchronize()
    dist.barrier()
    clk = clocks.stop()
    t_total_ms = float(times[:, 0].sum())
    t_total_ms = dist.max(t_total_ms)
    ms_per_step = t_total_ms / steps
    value = dist.sum(n * steps) / (t_total_ms / 1e3)

    # results and per-patch statistics of the last step
    err = rb.collect()
    nfail = int((err < 0).sum())
    stats = [cg.getsolverstats(i, 1) for i in ire]
    res_it = [cg.getiterationcounts(i, 1) for i in ire]
    t0 = min(s["t_start_ns"] for s in stats)
    ic_ms = float(times[-1, 2])
    lat_ms = np.array([(s["t_end_ns"] - t0) / 1e6 for s in stats]) + ic_ms
    # algorithmic bytes of the patch-solve kernels in one step: convolution traffic counted in
    # the kernel, plus the vector passes of the iterations (8 N bytes per pass):
    # NormCG 12 passes / iteration, GDsteady 20 / iteration + 16 / line-search step
    alg = 0.0
    for c, s, r in zip(cases, stats, res_it):
        npot = int(c["potprm"][0]) * int(c["potprm"][1])
        itgd = r["itgs"] if r["solver"] == 7 else 0
        alg += s["conv_bytes"] + 8.0 * npot * (12 * r["itcg"] + 20 * itgd + 16 * s["nls"])
    solve_ms = ms_per_step
    sm_cycles = float(sum(s["t_total"] for s in stats))
    # where the patch-solve kernel's time goes: SM cycles per phase summed over the patches
    # (phases nest: convolutions inside NORM and TANG, FP32 convolutions inside convolutions,
    # row scans inside the line search)
    phase_names = ("t_norm", "t_tang", "t_conv", "t_conv32", "t_ls", "t_scan", "t_diag", "t_gs")
    phases = {k[2:]: float(sum(s[k] for s in stats)) / max(sm_cycles, 1.0) for k in phase_names}
    n_fallback = int(sum(1 for s in stats if s["t_gs"] > 0))
    kernels_per_pass = int(round(times[-1, 3]))
    graph_sets = rb.graphs()
    peak, peak_kind = measured_peaks()
    fmap = cg.fma_peaks()
    achieved = alg / (solve_ms / 1e3) / 1e9
    rb.release()

    # end to end: one cntc_calculate_batch of the whole workload from host buffers (copies
    # inside the timed region).  The kernels are warm from the resident steps; this first
    # call of the batch path also allocates the library's staging arena (about a second),
    # which a separate warm-up call would cost a whole extra step to exclude.
    e2e_steps = 1
    dist.barrier()
    torch.cuda.synchronize()
    te = time.perf_counter()
    for _ in range(e2e_steps):
        e_err = cg.calculate_batch(ire, icp)
    torch.cuda.synchronize()
    te = dist.max(time.perf_counter() - te)
    e2e_value = dist.sum(n * e2e_steps) / te
    h2d_bytes, d2h_bytes = cg.lastcopybytes()
    # plain FP64 form on a sample of the same workload
    plain = None
    if args.plain_sample > 0:
        pc = [dict(c, mixed=0) for c in cases[:args.plain_sample]]
        pire = ire[:len(pc)]
        picp = [2] * len(pc)
        for i, c in zip(pire, pc):
            cg.setup_case(i, 2, c)
        prb = cg.ResidentBatch(pire, picp)
        pt = prb.solve(1)
        prb.collect()
        prb.release()
        mrb = cg.ResidentBatch(ire[:args.plain_sample], icp[:args.plain_sample])
        mt = mrb.solve(1)
        mrb.collect()
        mrb.release()
        mixed_sample_ms = float(mt[0, 0])
        # errors of the mixed form against the FP64 form on the same patches
        errs = form_errors(cg, pire, 1, 2, [c["fstat"] for c in pc])
        ferr = errs["ft"]
        # the per-call FP64 drop-in (one cntc_calculate per patch, one CTA each): the sum of the
        # patches' own solve times, measured in SM cycles by each patch's CTA in this pass (an
        # upper bound: there two CTAs share an SM)
        mhz = clk["sm_mhz"] if clk and clk.get("sm_mhz") else 2070.0
        cta_s = sum(cg.getsolverstats(i, 2)["t_total"] for i in pire) / (mhz * 1e6)
        plain = {"patches": len(pc), "solves_per_s": len(pc) / (float(pt[0, 0]) / 1e3),
                 "per_call_solves_per_s": len(pc) / cta_s,
                 "mixed_solves_per_s_same_sample": len(pc) / (mixed_sample_ms / 1e3),
                 "mixed_force_rel_err": {"max": float(ferr.max()), "p99": float(np.percentile(ferr, 99)),
                                         "median": float(np.median(ferr)), "above_1e-8": int((ferr > 1e-8).sum())},
                 "mixed_err_vs_fp64": summarize_errors(errs),
                 "note": "first %d patches of the workload, eps 1e-8, FP64 throughout, batched (solves_per_s) and "
                         "as per-call drop-in (per_call_solves_per_s: patches / sum of each patch's single-CTA "
                         "solve time in that pass); force error = |dF_t| / max(|F_t|, 1e-3 mu Fn) of the mixed "
                         "form against this FP64 form" % len(pc)}
    cpu = None
    small = None
    if dist.rank == 0 and not args.no_cpu_baseline:
        rate, thr, desc, _ = cpu_sample_rate(cases, args.seed, threads=args.cpu_threads or None)
        cpu = {"value": rate, "unit": UNIT, "cores": thr, "kind": "port", "sample": desc}
        small = small_patch_latency(cg)
    if dist.rank != 0:
        return None
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": dist.world, "steps": steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
        "steps_requested": args.steps,
        "config": {"workload": "batched mixed-size Hertzian steady rolling, %d patches, sides 24-160, "
                               "GDsteady, FP32 convolutions + FP64 refinement, eps 1e-8" % n,
                   "patches": n, "seed": args.seed, "parallelism": "replicas x%d" % dist.world,
                   "passes": "overlapped over %d buffer sets, each pass one CUDA graph replay (%d of %d sets "
                             "captured): influence coefficients, spectra, one persistent solve launch"
                             % (args.depth, graph_sets, args.depth),
                   "l2": "inputs larger than L2 (%.1f GB of io blocks alone)" % (d2h_bytes / 1e9)},
        "latency_ms": {"p50": float(np.percentile(lat_ms, 50)), "p99": float(np.percentile(lat_ms, 99)),
                       "definition": "completion time of each patch since the start of its step (batched)"},
        "failed_patches": nfail,
        "sm_gcycles_per_step": sm_cycles / 1e9,
        "phase_share_of_sm_cycles": phases,
        "steadygs_fallbacks": n_fallback,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": alg * TRAFFIC_PER_ALG_BYTE, "algorithmic_bytes": alg,
                     "traffic_unit": "bytes per launch", "kernel": "k_solve",
                     "kernels_per_step": kernels_per_pass, "peak_source": peak_kind,
                     "traffic_source": "DRAM bytes per algorithmic byte of one ncu capture of k_solve on 304 "
                                       "patches with sides <= 64 (41.5 GB for 71.4 GB algorithmic), times this "
                                       "launch's algorithmic bytes: an estimate",
                     "note": "k_solve is bound by the FP64 pipe (57.5 % of the active cycles with two CTAs per SM, "
                             "ncu on 304 patches), not by HBM; achieved = algorithmic bytes (convolution inputs, "
                             "spectra and outputs, and the iterations' vector passes) / patch-solve kernel time"},
        "fma_peaks": dict(fmap, note="FMA-chain peaks of this GPU timed with CUDA events on all SMs; k_solve's "
                                   "FP64 pipe is 57.5 % active with two CTAs per SM (ncu on 304 patches)"),
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d_bytes, "d2h_bytes_per_step": d2h_bytes,
                "errors": int((np.asarray(e_err) < 0).sum()),
                "note": "one cntc_calculate_batch call, including the first-call allocation of its staging arena"},
        "plain_fp64": plain,
        "small_patch": small,
        "clocks": clk,
        "gpu_launches": int(gpu_launches),
    }
    return out


# ------------------------------------------------------------------------------------------
# reference arm: the CPU oracle on the host cores
# ------------------------------------------------------------------------------------------
def run_reference(args, dist):
    """The reference arm: the oracle (the CPU restatement of the reference's solve path; the
    reference itself does not build here) on all host threads.  A warm-up step solves one small
    patch per thread; each timed step solves one stratified sample of the workload (one patch
    per size stratum, as many strata as threads)."""
    if dist.rank != 0:
        return None
    import pyoracle as po
    po.build()
    cases = workload(args.patches, args.seed, mixed=0)
    if args.cpu_max_side > 0:
        cases = [c for c in cases if max(c["potprm"][0], c["potprm"][1]) <= args.cpu_max_side]
    threads = args.cpu_threads or os.cpu_count() or 1
    small = [c for c in cases if c["potprm"][0] * c["potprm"][1] <= 48 * 48][:threads]
    from concurrent.futures import ThreadPoolExecutor
    for _ in range(args.warmup):
        with ThreadPoolExecutor(max_workers=threads) as ex:
            list(ex.map(lambda c: C.oracle_solve(dict(c, mixed=0), fast=True), small))
    tot_patch_s, tot_n, walls = 0.0, 0, []
    desc = ""
    for s in range(args.steps):
        r, thr, desc, wall = cpu_sample_rate(cases, args.seed + 7919 * s, threads=threads)
        n = len(stratified_sample(cases, threads, args.seed + 7919 * s))
        tot_patch_s += thr * n / r
        tot_n += n
        walls.append(wall)
    value = threads * tot_n / tot_patch_s
    desc = ("%d steps x %d patches, each step one stratified sample (one patch per equal-count stratum of element "
            "count over the full 24-160 side range, no extrapolation) solved by the oracle's baseline build on %d "
            "threads; rate = threads x patches / sum of per-patch seconds" % (args.steps, threads, threads))
    return {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": dist.world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": float(np.mean(walls)) * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
        "config": {"workload": "batched mixed-size Hertzian steady rolling, %d patches, sides 24-160, "
                               "GDsteady, FP64, eps 1e-8" % len(cases), "patches": len(cases), "seed": args.seed},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": desc},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


# ------------------------------------------------------------------------------------------
# serving stream: wheels x 2 patches, each patch a fixed grid (32..128 square), creepages and
# Fn on seeded random walks, every time step warm-started from the patch's previous traction;
# requests arrive as a Poisson stream and are served by cntc_calculate_async / cntc_wait
# ------------------------------------------------------------------------------------------
def serving_cases(wheels, seed):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(2 * wheels):
        m = int(rng.integers(32, 129))
        a = float(np.exp(rng.uniform(math.log(2.0), math.log(10.0))))
        b = float(np.exp(rng.uniform(math.log(2.0), math.log(10.0))))
        out.append(dict(tang=3, norm=1, bound=0, gausei=5, maxgs=999, maxin=100, maxnr=30, maxout=1, eps=1e-8,
                        poiss=C.NU_STEEL, gg=C.G_STEEL, fstat=float(rng.uniform(0.2, 0.4)), veloc=10000.0,
                        fn=float(rng.uniform(20e3, 150e3)), cksi=float(rng.uniform(-0.005, 0.005)),
                        ceta=float(rng.uniform(-0.005, 0.005)), cphi=float(rng.uniform(-0.5, 0.5)) * 1e-3,
                        ipotcn=-3, potprm=[m, m, a, b, 1.1], mixed=MIXED_TIER, iestim=1))
    return out, rng


def run_serving(args, dist):
    import torch
    import contact_gb300 as cg
    torch.cuda.set_device(dist.local)
    cg.load()
    cases, rng = serving_cases(args.wheels, 3)
    npatch = len(cases)
    for i, c in enumerate(cases):
        cg.setup_case(i + 1, 1, c)
    # first solve of every patch (cold start) through the batched path
    cg.calculate_batch(list(range(1, npatch + 1)), [1] * npatch)
    rate = args.rate
    total = npatch * args.time_steps
    steps_done = [0] * npatch
    free = list(range(npatch))
    lat, lock = [], threading.Lock()
    cv = threading.Condition(lock)
    inflight = [0]

    def waiter(i):
        ierr, l = cg.wait(i + 1, 1, with_latency=True)
        with cv:
            lat.append((l, ierr))
            inflight[0] -= 1
            free.append(i)
            cv.notify_all()

    t0 = time.perf_counter()
    t_next = t0
    submitted = 0
    threads = []
    while submitted < total:
        t_next += rng.exponential(1.0 / rate)
        now = time.perf_counter()
        if t_next > now:
            time.sleep(t_next - now)
        with cv:
            cv.wait_for(lambda: len(free) > 0)
            cand = [i for i in free if steps_done[i] < args.time_steps]
            if not cand:
                cv.wait_for(lambda: any(steps_done[i] < args.time_steps for i in free))
                cand = [i for i in free if steps_done[i] < args.time_steps]
            i = cand[int(rng.integers(len(cand)))]
            free.remove(i)
            inflight[0] += 1
        c = cases[i]
        c["cksi"] = float(np.clip(c["cksi"] + rng.normal(0, 2e-4), -0.005, 0.005))
        c["ceta"] = float(np.clip(c["ceta"] + rng.normal(0, 2e-4), -0.005, 0.005))
        c["fn"] = float(np.clip(c["fn"] + rng.normal(0, 2e3), 20e3, 150e3))
        cg.setcreepages(i + 1, 1, c["cksi"], c["ceta"], c["cphi"])
        cg.setnormalforce(i + 1, 1, c["fn"])
        steps_done[i] += 1
        assert cg.calculate_async(i + 1, 1) == 0
        th = threading.Thread(target=waiter, args=(i,), daemon=True)
        th.start()
        threads.append(th)
        submitted += 1
    for th in threads:
        th.join()
    wall = time.perf_counter() - t0
    ls = np.array([l for l, _ in lat])
    errs = sum(1 for _, e in lat if e < 0)
    if dist.rank != 0:
        return None
    return {"metric": METRIC, "value": total / wall, "unit": UNIT, "n_gpus": dist.world, "steps": args.time_steps,
            "warmup": 1, "ms_per_step": wall * 1e3 / args.time_steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic", "mode": "serving",
            "config": {"workload": "serving stream: %d wheels x 2 patches, grids 32..128 square, random-walk "
                                   "creepages (2e-4) and Fn (2 kN), warm start, Poisson arrivals at %.1f/s, "
                                   "admission budget 40 GB, %d time steps per patch" % (args.wheels, rate,
                                                                                        args.time_steps),
                       "requests": total},
            "latency_ms": {"p50": float(np.percentile(ls, 50) * 1e3), "p99": float(np.percentile(ls, 99) * 1e3),
                           "definition": "queueing to completion of each request"},
            "failed_requests": errs}


# ------------------------------------------------------------------------------------------
# large single patch (1024^2 rough surface), solved by a cooperative group of CTAs: FP64
# against mixed precision, time per solve, and the HBM roofline of the convolution phases
# (algorithmic bytes of the convolutions over the SM cycles spent in them at the sampled clock)
# ------------------------------------------------------------------------------------------
def run_large(args, dist):
    import torch
    import contact_gb300 as cg
    torch.cuda.set_device(dist.local)
    cg.load()
    m = args.large_side
    if m == 1024:
        base = C.config4(maxgs=args.large_maxgs, eps=args.large_eps)
    else:
        base = C.config1(m, maxgs=args.large_maxgs, eps=args.large_eps)
    forms = {}
    clocks = ClockSampler(dist.local)
    clocks.start()
    for mixed in (MIXED_TIER, 0):
        icp = 1 if mixed else 2
        cg.setup_case(1, icp, dict(base, mixed=mixed))
        rb = cg.ResidentBatch([1], [icp])
        if rb.setup_errors[0] != 0:
            raise RuntimeError("large patch could not be prepared")
        if args.warmup > 0:
            rb.solve(args.warmup)
        k0 = cg.kernel_launches()
        t = rb.solve(max(1, args.steps))
        launches = cg.kernel_launches() - k0
        err = rb.collect()
        rb.release()
        st = cg.getsolverstats(1, icp)
        it = cg.getiterationcounts(1, icp)
        forms[mixed] = dict(ms=float(t[:, 0].mean()), ierror=int(err[0]), stats=st, it=it, res=cg.results(1, icp),
                            launches=launches)
    clk = clocks.stop()
    # end to end through cntc_calculate (host buffers; copies and set-up inside)
    torch.cuda.synchronize()
    te = time.perf_counter()
    e_err = cg.calculate(1, 1)
    te = time.perf_counter() - te
    h2d, d2h = cg.lastcopybytes()
    a, b = forms[MIXED_TIER], forms[0]
    ft = math.hypot(b["res"]["fx"], b["res"]["fy"])
    ferr = math.hypot(a["res"]["fx"] - b["res"]["fx"], a["res"]["fy"] - b["res"]["fy"]) / max(ft, 1e-300)
    mhz = clk.get("sm_mhz") or 2070.0
    peak, peak_kind = measured_peaks()

    def conv_roof(f):
        s = f["stats"]
        t_s = s["t_conv"] / (mhz * 1e6)
        return s["conv_bytes"] / max(t_s, 1e-12) / 1e9

    if dist.rank != 0:
        return None
    ach = conv_roof(a)
    return {"metric": METRIC, "value": 1e3 / a["ms"], "unit": UNIT, "n_gpus": dist.world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": a["ms"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic", "mode": "large",
            "config": {"workload": ("large single patch %dx%d, rough surface (seed 4), Fn 150 kN, creepages "
                                    "(0.003, 0, 0.3 rad/m), mu 0.25" % (m, m) if m == 1024 else
                                    "grid-sweep patch %dx%d, rough surface (seed 1), Fn 100 kN, creepages "
                                    "(0.002, 0.001, 0.2 rad/m), mu 0.3" % (m, m)) +
                                   ", GDsteady eps %g, maxgs %d; one patch group of %d CTAs" % (
                                       args.large_eps, args.large_maxgs, int(a["stats"]["ctas"])),
                       "l2": "inputs larger than L2 (io block %.2f GB; work area about 1 GB)" % (h2d / 1e9)},
            "fp64_solves_per_s": 1e3 / b["ms"],
            "mixed_vs_fp64": {"force_rel_err": ferr,
                              "fn_rel_err": abs(a["res"]["fn"] - b["res"]["fn"]) / b["res"]["fn"],
                              "pmax_rel_err": abs(a["res"]["pmax"] - b["res"]["pmax"]) / b["res"]["pmax"],
                              "eldiv_differences": int((a["res"]["igs"] != b["res"]["igs"]).sum()),
                              "traction_max_err_over_pmax": float(max(np.abs(a["res"][k] - b["res"][k]).max()
                                                                      for k in ("pn", "px", "py")) / b["res"]["pmax"])},
            "iterations": {"mixed": a["it"], "fp64": b["it"], "ierror": [a["ierror"], b["ierror"]]},
            "phase_share_of_sm_cycles": {k[2:]: a["stats"][k] / a["stats"]["t_total"] for k in
                                         ("t_norm", "t_tang", "t_conv", "t_conv32", "t_ls", "t_scan", "t_diag")},
            "roofline": {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                         "traffic": None, "kernel": "k_solve convolution phases (patch group)",
                         "fp64_form_achieved": conv_roof(b), "peak_source": peak_kind,
                         "note": "algorithmic bytes of the convolutions / SM cycles in them at the sampled clock"},
            "e2e": {"value": 1.0 / te, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "ierror": int(e_err)},
            "clocks": clk, "gpu_launches": int(a["launches"])}


# ------------------------------------------------------------------------------------------
# the reference's performance inputs (perfc_test/*.inp, committed in parsed form): each case
# solved in FP64 through cntc_calculate (host buffers, set-up and copies included), against
# the counts and wall-clock seconds of the reference's published run (1 thread, 2016)
# ------------------------------------------------------------------------------------------
def run_perfc(args, dist):
    import torch
    import contact_gb300 as cg
    from contact_gb300 import inp
    torch.cuda.set_device(dist.local)
    cg.load()
    with open(os.path.join(ROOT, "tests", "golden", "perfc_cases.json")) as f:
        gold = json.load(f)["cases"]
    rows = []
    # one warm-up solve (kernel attributes, streams); every timed problem is new, so it
    # computes its influence coefficients like the reference's single run
    cg.setup_case(199, 1, inp.materialize(gold[0]["case"]))
    cg.calculate(199, 1)
    cg.finalize(199)
    def timed(ire, case):
        cg.setup_case(ire, 2, case)
        torch.cuda.synchronize()
        t = time.perf_counter()
        ierr = cg.calculate(ire, 2)
        torch.cuda.synchronize()
        return ierr, time.perf_counter() - t

    for k, g in enumerate(gold):
        case = inp.materialize(g["case"])
        ire = 200 + k
        ierr, dt = timed(ire, case)
        r = cg.results(ire, 2)
        ref = g["reference"]
        row = {"name": g["name"], "grid": case["potprm"][:2], "ierror": ierr, "s": dt, "ref_s": ref["wall_s"],
               "speedup": ref["wall_s"] / dt if dt > 0 else None, "ctas": int(cg.getsolverstats(ire, 2)["ctas"])}
        # the launch shape tuned per size class (CNTC_if_groupctas = -1): the first call of a
        # class times both shapes, so a warm-up call on another problem precedes the timed one
        tcase = dict(case, group=-1)
        timed(400 + k, tcase)
        cg.finalize(400 + k)
        ierr_t, dt_t = timed(600 + k, tcase)
        row.update(s_tuned=dt_t, speedup_tuned=ref["wall_s"] / dt_t if dt_t > 0 else None,
                   ctas_tuned=int(cg.getsolverstats(600 + k, 2)["ctas"]), ierror_tuned=ierr_t)
        cg.finalize(600 + k)
        if "ncon" in ref:
            row.update(ncon=r["ncon"], itcg=r["itcg"], ref_ncon=ref["ncon"], ref_itcg=ref["itcg"])
        else:
            row.update(nslip=r["nslip"], itcg=r["itgs"], ref_nslip=ref["nslp"], ref_itcg=ref["itgs"])
        rows.append(row)
        cg.finalize(ire)
    if dist.rank != 0:
        return None
    tot, tot_ref = sum(r["s"] for r in rows), sum(r["ref_s"] for r in rows)
    tot_tuned = sum(r["s_tuned"] for r in rows)
    return {"metric": METRIC, "value": len(rows) / tot, "unit": UNIT, "n_gpus": dist.world, "steps": 1,
            "warmup": 1, "ms_per_step": tot * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "the reference's performance inputs (perfc_test)", "mode": "perfc",
            "config": {"workload": "perfc_test normal problems 1p-8p, 1f-4f and shift problems 1s-8s, FP64, "
                                   "one cntc_calculate each; s: default launch shape, s_tuned: the shape "
                                   "tuned per size class (CNTC_if_groupctas = -1)"},
            "total_s": tot, "total_s_tuned": tot_tuned, "reference_total_s": tot_ref, "cases": rows}


# ------------------------------------------------------------------------------------------
# accuracy of the forms on a sample of the batched workload: the mixed and the FP64 form at the
# workload's tolerance and at a tight one, each against the others
# ------------------------------------------------------------------------------------------
def run_accuracy(args, dist):
    import torch
    import contact_gb300 as cg
    torch.cuda.set_device(dist.local)
    cg.load()
    n = args.plain_sample
    cases = workload(n, args.seed)
    ire = list(range(1, n + 1))
    eps = cases[0]["eps"]
    forms = {1: ("mixed", eps, {}), 2: ("fp64", eps, {"mixed": 0}),
             3: ("fp64", args.tight_eps, {"mixed": 0, "eps": args.tight_eps}),
             4: ("mixed", args.tight_eps, {"eps": args.tight_eps})}
    rates, iters = {}, {}
    for icp, (name, e, over) in forms.items():
        for i, c in zip(ire, cases):
            cg.setup_case(i, icp, dict(c, **over))
        rb = cg.ResidentBatch(ire, [icp] * n)
        t = rb.solve(1)
        rb.collect()
        rb.release()
        key = "%s_eps%g" % (name, e)
        rates[key] = n / (float(t[0, 0]) / 1e3)
        iters[key] = float(np.mean([cg.getiterationcounts(i, icp)["itgs"] for i in ire]))
    fstat = [c["fstat"] for c in cases]
    pairs = {"mixed_vs_fp64_same_eps": (1, 2), "fp64_eps_vs_fp64_tight": (2, 3),
             "mixed_eps_vs_fp64_tight": (1, 3), "mixed_tight_vs_fp64_tight": (4, 3)}
    errs = {k: form_errors(cg, ire, a, b, fstat) for k, (a, b) in pairs.items()}
    table = {k: summarize_errors(v) for k, v in errs.items()}
    # the patches where mixed and FP64 differ most at the workload's eps, with the distance of
    # each form from the tightly converged FP64 answer
    worst = []
    for k in np.argsort(-errs["mixed_vs_fp64_same_eps"]["ft"])[:8]:
        worst.append({"patch": int(k), "grid": cases[k]["potprm"][:2],
                      "ft_mixed_vs_fp64": float(errs["mixed_vs_fp64_same_eps"]["ft"][k]),
                      "ft_fp64_vs_tight": float(errs["fp64_eps_vs_fp64_tight"]["ft"][k]),
                      "ft_mixed_vs_tight": float(errs["mixed_eps_vs_fp64_tight"]["ft"][k]),
                      "ft_mixed_tight_vs_tight": float(errs["mixed_tight_vs_fp64_tight"]["ft"][k])})
    if dist.rank != 0:
        return None
    return {"metric": METRIC, "value": rates["mixed_eps%g" % eps], "unit": UNIT, "n_gpus": dist.world,
            "steps": 1, "warmup": 0, "ms_per_step": n / rates["mixed_eps%g" % eps] * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
            "data": "synthetic", "mode": "accuracy",
            "config": {"workload": "first %d patches of the batched workload (seed %d), mixed tier %d and FP64, "
                                   "at eps %g and at eps %g" % (n, args.seed, MIXED_TIER, eps, args.tight_eps)},
            "solves_per_s": rates, "mean_gd_iterations": iters, "errors": table, "worst_patches": worst}


def main():
    args = parse()
    dist = Dist()
    try:
        if args.serving and args.impl != "reference":
            out = run_serving(args, dist)
        elif args.large and args.impl != "reference":
            out = run_large(args, dist)
        elif args.perfc and args.impl != "reference":
            out = run_perfc(args, dist)
        elif args.accuracy and args.impl != "reference":
            out = run_accuracy(args, dist)
        else:
            out = run_reference(args, dist) if args.impl == "reference" else run_gb300(args, dist)
        if out is not None:
            print(json.dumps(out), flush=True)
    finally:
        dist.close()


if __name__ == "__main__":
    main()
