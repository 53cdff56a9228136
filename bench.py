#!/usr/bin/env python3
"""Newton steps/s of the THCM ocean continuation on one GB300.

Workload (default ``global_96x38x12``): the 4-degree global ocean, 96x38x12
cells with a seeded land mask (about 30% land, periodic in longitude), 262,656
unknowns. A steady state at Combined Forcing ``--setup-comb`` is computed first
(untimed); then ``--warmup`` pseudo-arclength continuation steps in the
freshwater forcing ("Salinity Forcing", par 15) run untimed and ``--steps``
steps are timed, first on the mixed path (FP32 factors, FP64 GMRES and
Newton: IEMIC_PREC_MIXED), then from the same point on the plain FP64 path.
Every linear solve reaches ||b - J x|| <= 1e-8 ||b|| and every corrector
||F(x)||_2 <= 1e-8 ||F(0)||_2 (the reference's residual test 'R').

A "step" is one continuation step (predictor plus Newton corrector); the
metric counts Newton corrector iterations (one Jacobian, three residuals,
one preconditioner rebuild, the bordered solve(s) and the update each) per
second of device time. ``--impl reference`` times the CPU restatement of the same
Newton iteration (C++ oracle assembly + numpy/LAPACK multifrontal LU) on the
host cores; it is the CPU baseline, not the target. The reference arm
(`--impl reference`) runs the CPU port of the same continuation (restated
driver, oracle assembly, FP64 multifrontal LU with the reference's
once-per-step preconditioner) from the committed CPU start state
tests/golden/start_global96.npz, for at most --ref-steps steps.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(REPO, "i-emic_gb300"))

METRIC = "Newton steps/s, 96×38×12 ocean, to 1e-8 residual: FP32+refine vs FP64 GPU"
UNIT = "Newton steps/s"
# Preconditioner policy of both arms (iemic_continuation_opts.refactor_each_newton = 2):
# once per continuation step as in Ocean::preProcess, plus a rebuild on the
# current Jacobian once the Krylov time a factorisation costs beyond its first
# solve exceeds the factorisation's own time.
REFACTOR = 2


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="global_96x38x12", choices=["global_96x38x12", "box_16x16x4"])
    ap.add_argument("--setup-comb", type=float, default=0.1)
    ap.add_argument("--fp64-steps", type=int, default=None, help="continuation steps of the FP64 comparison")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true", help="skip the host-buffer end-to-end run")
    ap.add_argument("--cpu-iters", type=int, default=1, help="Newton iterations of the CPU sample")
    ap.add_argument("--ref-steps", type=int, default=2,
                    help="continuation steps the reference arm (CPU port) times at most")
    ap.add_argument("--dt", type=float, default=0.05, help="transient: time step of the theta method")
    ap.add_argument("--mode", default="continuation", choices=["continuation", "newton1", "newton_large", "transient"],
                    help="newton1: one Newton iteration per precision from the seeded state, per-kernel-class "
                         "device times (a short case for profiling); newton_large: Newton iterations on the "
                         "360x160x20 ocean with per-kernel HBM rates")
    ap.add_argument("--large-steps", type=int, default=5, help="timed Newton iterations of newton_large")
    ap.add_argument("--subst-threshold", type=int, default=None,
                    help="newton_large: largest front kept as whole inverses (default: the library's)")
    return ap.parse_args()


def workload(name):
    from iemic import workloads as W
    if name == "global_96x38x12":
        cfg = W.global_96x38x12()
        return cfg, W.seeded_global_mask(cfg, 0), None
    cfg = W.box_16x16x4()
    return cfg, None, W.box_forcing(cfg)


def continuation_opts(ocean, precision, steps, fscale):
    """Freshwater-forcing continuation with the reference's test settings
    (test/ocean/continuation_params.xml: step sizes 1e-2 / 1e-8 / 1e-1, 15
    Newton iterations, epsilon 1e-5, secant tangent, Newton-chord hybrid,
    predictor bound 3000) and the corrector converged to
    ||F||_2 <= 1e-8 ||F(0)||_2 (residual test 'R')."""
    return ocean.default_continuation_opts("Salinity Forcing", precision), dict(
        ds=0.01, ds_min=1e-8, ds_max=0.1, destination=10.0, max_steps=steps, max_newton=15, min_newton=1,
        opt_newton=3.5, newton_tol=1e-8 * fscale, residual_test=b"R", normalize=b"N", tangent=b"S",
        newton_chord=1, epsilon=1e-5, predictor_bound=3000.0, tan_scaling=1.0, refactor_each_newton=REFACTOR)


def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group("nccl")
    return rank, world


def _all_reduce(value, world, op_name):
    """Replica aggregation over the process group (NCCL on GPUs, gloo on CPU)."""
    if world == 1:
        return value
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([value], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=getattr(dist.ReduceOp, op_name))
    return float(t.item())


def barrier_max(value, world):
    """Max over ranks: the timed region ends when the slowest replica ends."""
    return _all_reduce(value, world, "MAX")


def barrier_sum(value, world):
    """Sum over ranks: the work all replicas did."""
    return _all_reduce(value, world, "SUM")


class Clocks:
    """nvidia-smi samples during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.p = None
        try:
            self.p = subprocess.Popen(["nvidia-smi", "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                                       "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return None
        self.p.terminate()
        try:
            out, _ = self.p.communicate(timeout=10)
        except subprocess.TimeoutExpired:
            self.p.kill()
            out, _ = self.p.communicate()
        dev = os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0]
        sm, smax, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            if dev.isdigit() and f[0] != dev and len(set(l.split(",")[0] for l in out.splitlines())) > 1:
                continue
            try:
                sm.append(float(f[1]))
                smax = max(smax, float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def roofline(stats, peaks):
    """Roofline of the dominant instrumented kernel class in the timed region."""
    counted = {k: v for k, v in stats.items() if k in ("factor_gemm", "solve_gemv", "assembly", "spmv")}
    name, s = max(counted.items(), key=lambda kv: kv[1]["ms"])
    avg_ms = s["ms"] / max(s["launches"], 1)
    out = {"kernel": name, "launches": s["launches"], "avg_launch_ms": avg_ms}
    if name == "factor_gemm":
        # FP32 (or FP64) SIMT GEMM: no measured SIMT peak exists; nominal FP32 rate
        peak = 2 * 128 * 152 * peaks.get("sm_max_mhz", 2070.0) * 1e6 / 1e12
        ach = s["flops"] / max(s["launches"], 1) / (avg_ms * 1e-3) / 1e12
        out.update(bound="fp32_simt", achieved=ach, peak=peak, unit="TFLOP/s", frac=ach / peak,
                   peak_source="nominal FP32 SIMT (152 SMs x 128 FMA/clk x max clock)")
    else:
        peak = peaks.get("hbm_gbs", 6800.0)
        ach = s["bytes"] / max(s["launches"], 1) / (avg_ms * 1e-3) / 1e9
        out.update(bound="hbm", achieved=ach, peak=peak, unit="GB/s", frac=ach / peak,
                   peak_source="measured" if "hbm_gbs" in peaks else "fallback")
    out["algorithmic_bytes_per_launch"] = s["bytes"] / max(s["launches"], 1)
    out["traffic"] = None
    tf = os.path.join(REPO, "profiles", "traffic_%s.json" % name)
    if os.path.exists(tf):
        try:
            with open(tf) as fh:
                out["traffic"] = json.load(fh).get("dram_bytes_per_launch")
        except (OSError, ValueError):
            pass
    out["classes"] = {k: {"ms": v["ms"], "launches": v["launches"]} for k, v in stats.items()}
    out["timing"] = ("CUDA events around every launch on the launching stream, in an instrumented repeat of "
                     "the timed mixed steps from the same starting point")
    return out


def arm_summary(r):
    """Progress and cost of one timed arm: steps taken and failed, the
    parameter reached, solves that stopped above tolerance, and the accepted
    continuation steps per second next to the Newton-iteration rate."""
    st = r["stats"]
    acc = st["steps"] - st["failed_steps"]
    out = {k: st[k] for k in ("steps", "failed_steps", "newton_iters", "linear_solves", "unconverged_solves",
                              "krylov_iters", "factorizations", "par", "time_assembly_ms", "time_factor_ms",
                              "time_solve_ms")}
    out.update(value=r["value"], ms=r["ms"], accepted_steps=acc,
               continuation_steps_per_s=acc / (r["ms"] * 1e-3))
    return out


def load_peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as fh:
            return json.load(fh)
    except (OSError, ValueError):
        return {}


# ---------------------------------------------------------------------------
# CPU baseline: the oracle's Newton iteration on the host cores
# ---------------------------------------------------------------------------
def cpu_newton_sample(cfg, lm, frc, iters, par_setup):
    """One (or more) Newton corrector iterations on the CPU: oracle assembly of
    J and F (plus F(par+eps) for dF/dpar), FP64 multifrontal LU, two solves and
    the update, from the seeded rest state at the workload's parameters."""
    import oracle
    from oracle.multifrontal import Factorization, Plan
    from iemic import workloads as W
    o = oracle.Oracle(cfg, lm)
    if frc:
        o.set_forcing(**frc)
    names = {"Combined Forcing": "COMB", "Temperature Forcing": "TEMP", "Salinity Forcing": "SALT",
             "Wind Forcing": "WIND"}
    for name, v in W.STARTING_PARAMETERS:
        o.set_par(names[name], v)
    o.set_par("COMB", par_setup)
    plan = Plan(o.landm(), cfg["n"], cfg["m"], cfg["l"], cfg["periodic"])
    rp, ci = o.graph()
    x = W.rest_state_with_ts_noise(cfg, 0)
    eps = 1e-5
    salt = o.get_par("SALT")
    t0 = time.perf_counter()
    for _ in range(iters):
        F = o.rhs(x)
        o.set_par("SALT", salt + eps)
        dfdp = (o.rhs(x) - F) / eps
        o.set_par("SALT", salt)
        vals, _ = o.jacobian(x)
        fact = Factorization(plan, rp, ci, vals)
        fact.solve(dfdp)            # J y = dF/dpar (the bordered corrector's second solve)
        x = x + fact.solve(-F)
    dt = time.perf_counter() - t0
    o.close()
    threads = os.cpu_count()
    return {"value": iters / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": "%d Newton iteration(s) at %s: oracle assembly (J, F, F(par+eps)) + FP64 multifrontal LU "
                      "(numpy/OpenBLAS, %d threads) + 2 exact solves; %.1f s" % (iters, "C2" if cfg["n"] == 96
                                                                                   else "box", threads, dt)}


# ---------------------------------------------------------------------------
def workload_config(args, cfg, nd, par_start, fscale):
    """The workload description both arms print (computed the same way on
    the CPU and the GPU side, rounded so that the two agree)."""
    return {"workload": args.workload, "grid": [cfg["n"], cfg["m"], cfg["l"]], "unknowns": nd,
            "continuation_parameter": "Salinity Forcing", "setup_combined_forcing": args.setup_comb,
            "warmup_steps": args.warmup, "start_salinity_forcing": float("%.6g" % par_start),
            "linear_tol": 1e-8, "newton_tol_abs": float("%.6g" % (1e-8 * fscale)),
            "preconditioner_policy": "once per step + cost-balanced rebuilds",
            "parallelism": "replicas", "l2": "working set larger than L2 (factors of 1.5-3 GB per apply)"}


START_STATE = os.path.join(REPO, "tests", "golden", "start_global96.npz")


def cpu_continuation_sample(args, steps):
    """The CPU port of the timed continuation: the restated Continuation.H
    driver (oracle/continuation.py) with the bench's options on the restated
    THCM model (oracle C++ assembly), solves by the FP64 multifrontal LU on
    all host cores with the reference's preconditioner policy (a new
    factorisation once per continuation step, GMRES on it for the step's later
    Jacobians), from the committed CPU start state at the Salinity Forcing the
    GPU arm starts from. Returns (cpu_baseline dict, details) or None when the
    start state is not available for the workload."""
    import oracle
    from oracle.continuation import Continuation, MultifrontalModel
    from oracle.multifrontal import Plan
    from iemic import workloads as W
    if args.workload != "global_96x38x12" or not os.path.exists(START_STATE):
        return None
    cfg, lm, frc = workload(args.workload)
    st0 = np.load(START_STATE)
    o = oracle.Oracle(cfg, lm)
    names = {"Combined Forcing": "COMB", "Temperature Forcing": "TEMP", "Salinity Forcing": "SALT",
             "Wind Forcing": "WIND"}
    for name, v in W.STARTING_PARAMETERS:
        o.set_par(names[name], v)
    fscale = float(st0["fscale"])           # ||F(0)|| at the starting parameters, as the GPU arm uses
    o.set_par("COMB", float(st0["combined_forcing"]))
    par0 = float(st0["salinity_forcing"])
    o.set_par("SALT", par0)
    plan = Plan(o.landm(), cfg["n"], cfg["m"], cfg["l"], cfg["periodic"])
    M = MultifrontalModel(o, plan, policy="step")
    t0 = time.perf_counter()
    C = Continuation(M, st0["x"], par="SALT", ds=0.01, ds_min=1e-8, ds_max=0.1, destination=10.0, max_steps=steps,
                     max_newton=15, min_newton=1, opt_newton=3.5, newton_tol=1e-8 * fscale, residual_test="R",
                     normalize="N", tangent="S", newton_chord=True, epsilon=1e-5, predictor_bound=3000.0,
                     tan_scaling=1.0)
    st = C.run()
    dt = time.perf_counter() - t0
    nd = o.ndim
    o.close()
    cores = os.cpu_count()
    warm_note = "" if int(st0["warmup"]) == args.warmup else (
        " (the committed start state follows %d warm-up steps; this run asked for %d)" % (int(st0["warmup"]),
                                                                                         args.warmup))
    sample = ("%d continuation step(s) (%d Newton iterations, %d factorisations, %d GMRES iterations) from "
              "Salinity Forcing %.6g to %.6g: oracle assembly + FP64 multifrontal LU (numpy/OpenBLAS, %d threads), "
              "%.1f s%s" % (st["steps"], st["newton_iters"], M.factorizations, M.krylov, par0, C.par, cores, dt,
                           warm_note))
    base = {"value": st["newton_iters"] / dt, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample}
    return base, dict(cfg=cfg, nd=nd, par0=par0, fscale=fscale, st=st, dt=dt, par=C.par)


def run_reference(args, rank, world):
    """`--impl reference`: the CPU port of the same continuation
    (cpu_continuation_sample), at most --ref-steps continuation steps, on
    rank 0 only."""
    if rank != 0:
        return
    out = cpu_continuation_sample(args, max(1, min(args.steps, args.ref_steps)))
    if out is None:
        print(json.dumps({"impl": "reference", "unavailable": "the CPU start state of %s is not committed"
                          % args.workload}), flush=True)
        return
    base, d = out
    st = d["st"]
    value = base["value"]
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": st["steps"],
            "warmup": args.warmup, "ms_per_step": d["dt"] * 1e3 / max(st["steps"], 1), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded land mask, idealized forcing)",
            "config": workload_config(args, d["cfg"], d["nd"], d["par0"], d["fscale"]),
            "impl": "reference", "cpu_baseline": base, "newton_iters": st["newton_iters"],
            "arm_preconditioner_policy": "FP64 multifrontal LU rebuilt once per continuation step (Ocean::preProcess), "
                                         "GMRES(100) on it for the step's later Jacobians",
            "continuation": {"steps": st["steps"], "failed_steps": st["failed_steps"], "par": d["par"]},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args, rank, world):
    import ctypes

    import torch
    from iemic import Ocean, load_library
    from iemic import workloads as W
    from iemic.ocean import ContinuationStats, _asdict

    torch.cuda.init()
    L = load_library()
    cfg, lm, frc = workload(args.workload)
    oc = Ocean(cfg, lm, forcing=frc, starting_parameters=W.STARTING_PARAMETERS)
    nd = oc.ndim
    fscale = float(np.linalg.norm(oc.computeRHS(np.zeros(nd))))
    stream = torch.cuda.ExternalStream(oc.stream())

    # --- setup (untimed): steady state at Combined Forcing = setup_comb
    oc.setPar("Combined Forcing", 0.0)
    x0, st0 = oc.continuation(np.zeros(nd), par="Combined Forcing", precision=1, ds=args.setup_comb / 2,
                              ds_max=args.setup_comb, destination=args.setup_comb, max_steps=20,
                              newton_tol=1e-8 * fscale, residual_test=b"R", predictor_bound=1e30)
    if st0["status"] != 0 or not st0["reached_destination"]:
        raise RuntimeError("setup continuation failed: %s" % st0)

    def cont_dev(x_dev, precision, steps):
        o, kw = continuation_opts(oc, precision, steps, fscale)
        for k, v in kw.items():
            setattr(o, k, v)
        st = ContinuationStats()
        rc = L.iemic_continuation_run_dev(oc.handle, ctypes.c_void_p(x_dev.data_ptr()), ctypes.byref(o),
                                          ctypes.byref(st))
        s = _asdict(st)
        s["status"] = rc
        if rc != 0:
            raise RuntimeError("continuation failed: %s" % s)
        return s

    # --- warm-up: W continuation steps in the freshwater forcing (mixed path)
    salt0 = oc.getPar("Salinity Forcing")
    xw = torch.tensor(x0, dtype=torch.float64, device="cuda")
    if args.warmup > 0:
        cont_dev(xw, 1, args.warmup)
    par_w = oc.getPar("Salinity Forcing")
    x_start = xw.clone()

    peaks = load_peaks()
    info = oc.solverInfo()
    results = {}
    fp64_steps = args.steps if args.fp64_steps is None else args.fp64_steps
    arms = [("mixed", 1, args.steps)] + ([("fp64", 0, fp64_steps)] if fp64_steps > 0 else [])
    for label, prec, steps in arms:
        x = x_start.clone()
        oc.setPar("Salinity Forcing", par_w)
        torch.cuda.synchronize()
        if world > 1:
            import torch.distributed as dist
            dist.barrier()
        timing = label == "mixed"
        if timing:
            clocks = Clocks()
            n0 = L.iemic_launch_count()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        st = cont_dev(x, prec, steps)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        if timing:
            launches = L.iemic_launch_count() - n0
            clk = clocks.stop()
        ms = barrier_max(ms, world)
        iters = barrier_sum(st["newton_iters"], world)
        results[label] = dict(ms=ms, newton_iters=iters, stats=st, value=iters / (ms * 1e-3))
        if timing:
            results[label].update(launches=launches, clocks=clk)

    # --- per-kernel device times: the timed mixed steps repeated from the same
    # point with CUDA events around every launch (event nodes in the same
    # captured graphs, on the stream the kernels run on), so the timed region
    # above stays uninstrumented
    x = x_start.clone()
    oc.setPar("Salinity Forcing", par_w)
    oc.kernelTiming(True)
    cont_dev(x, 1, args.steps)
    torch.cuda.synchronize()
    results["mixed"]["kstats"] = oc.kernelStats()
    results["mixed"]["timing_failures"] = oc.kernelTimingFailures()
    oc.kernelTiming(False)

    # --- end to end through the public API with host buffers (mixed path)
    e2e = None
    if not args.no_e2e:
        xh = x_start.cpu().numpy()
        oc.setPar("Salinity Forcing", par_w)
        o, kw = continuation_opts(oc, 1, args.steps, fscale)
        kw["par"] = "Salinity Forcing"
        kw["precision"] = 1
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        _, ste = oc.continuation(xh, **kw)
        e2e_s = time.perf_counter() - t0
        e2e_iters = barrier_sum(ste["newton_iters"], world)
        e2e_s = barrier_max(e2e_s, world)
        e2e = {"value": e2e_iters / e2e_s, "unit": UNIT, "h2d_bytes_per_step": 8 * nd / args.steps,
               "d2h_bytes_per_step": 8 * nd / args.steps,
               "note": "one continuation call of %d steps with the state in host memory" % args.steps}

    if rank != 0:
        return
    mixed, fp64 = results["mixed"], results.get("fp64")
    line = {
        "metric": METRIC, "value": mixed["value"], "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": mixed["ms"] / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 factors / f64 Krylov+Newton",
        "data": "synthetic (seeded land mask, idealized forcing)",
        "config": workload_config(args, cfg, nd, par_w, fscale),
        "solver": {"factor_gb_fp32": 4e-9 * info["factor_entries"], "factor_gflop": info["factor_flops"] / 1e9,
                   "fronts": info["fronts"], "start_salinity_forcing": par_w, "initial_salinity_forcing": salt0},
        "newton_iters": mixed["newton_iters"], "continuation": arm_summary(mixed),
        "fp64_gpu": None if fp64 is None else arm_summary(fp64),
        "speedup_vs_fp64_gpu": None if fp64 is None else mixed["value"] / fp64["value"],
        "speedup_per_continuation_step": None if fp64 is None else
        (fp64["ms"] / max(fp64["stats"]["steps"] - fp64["stats"]["failed_steps"], 1)) /
        (mixed["ms"] / max(mixed["stats"]["steps"] - mixed["stats"]["failed_steps"], 1)),
        "e2e": e2e,
        "gpu_launches": mixed["launches"],
        "clocks": mixed["clocks"],
        "roofline": roofline(mixed["kstats"], peaks),
    }
    if world == 1 and not args.no_cpu_baseline:
        out = cpu_continuation_sample(args, 1)
        line["cpu_baseline"] = out[0] if out is not None else cpu_newton_sample(cfg, lm, frc, args.cpu_iters,
                                                                                  args.setup_comb)
    print(json.dumps(line), flush=True)


def run_newton1(args):
    """One Newton iteration (J, F, F(par+eps), preconditioner, two solves) per
    precision from the seeded rest state; per-kernel-class device times."""
    import torch
    from iemic import Ocean
    from iemic import workloads as W
    torch.cuda.init()
    cfg, lm, frc = workload(args.workload)
    oc = Ocean(cfg, lm, forcing=frc, starting_parameters=W.STARTING_PARAMETERS)
    oc.setPar("Combined Forcing", args.setup_comb)
    x = W.rest_state_with_ts_noise(cfg, 0)
    out = {"mode": "newton1", "workload": args.workload, "solver": oc.solverInfo()}
    for label, prec in (("mixed", 1), ("fp64", 0)):
        # pass 0 builds the plan and allocates; pass 1 times every kernel class
        # (the same graphs with event nodes); pass 2 runs untimed, as in production
        for rep in range(3):
            oc.kernelTiming(rep == 1)
            t0 = time.perf_counter()
            F = oc.computeRHS(x)
            oc.setPar("Salinity Forcing", oc.getPar("Salinity Forcing") + 1e-5)
            Fe = oc.computeRHS(x)
            oc.setPar("Salinity Forcing", oc.getPar("Salinity Forcing") - 1e-5)
            oc.computeJacobian(x)
            _, s1 = oc.solve((Fe - F) / 1e-5, precision=prec)
            _, s2 = oc.solve(-F, precision=prec)
            wall = time.perf_counter() - t0
            if rep == 1:
                ks = oc.kernelStats()
                failed = oc.kernelTimingFailures()
                timed = {"wall_s": wall, "solve1": s1, "solve2": s2}
            oc.kernelTiming(False)
        out[label] = {"wall_s": wall, "solve1": s1, "solve2": s2, "timed_pass": timed, "timing_failures": failed,
                      "classes_ms": {k: round(v["ms"], 3) for k, v in ks.items()},
                      "launches": {k: v["launches"] for k, v in ks.items()}}
    print(json.dumps(out), flush=True)


def run_transient(args):
    """Implicit time steps (theta = 1, ThetaModel<Ocean> + transient Newton)
    after a jump of the freshwater forcing: the steady state at Combined
    Forcing --setup-comb, Salinity Forcing raised by 0.1, then --warmup
    untimed and --steps timed steps of size --dt, per precision, through the
    public host-buffer API (state copied in and out every step)."""
    import torch
    from iemic import Ocean
    from iemic import workloads as W
    torch.cuda.init()
    cfg, lm, frc = workload(args.workload)
    oc = Ocean(cfg, lm, forcing=frc, starting_parameters=W.STARTING_PARAMETERS)
    nd = oc.ndim
    fscale = float(np.linalg.norm(oc.computeRHS(np.zeros(nd))))
    oc.setPar("Combined Forcing", 0.0)
    x0, st0 = oc.continuation(np.zeros(nd), par="Combined Forcing", precision=1, ds=args.setup_comb / 2,
                              ds_max=args.setup_comb, destination=args.setup_comb, max_steps=20,
                              newton_tol=1e-8 * fscale, residual_test=b"R", predictor_bound=1e30)
    if st0["status"] != 0 or not st0["reached_destination"]:
        raise RuntimeError("setup continuation failed: %s" % st0)
    oc.setPar("Salinity Forcing", oc.getPar("Salinity Forcing") + 0.1)
    out = {"mode": "transient", "workload": args.workload, "dt": args.dt, "theta": 1.0, "steps": args.steps,
           "warmup": args.warmup, "unknowns": nd}
    for label, prec in (("mixed", 1), ("fp64", 0)):
        x = x0.copy()
        for _ in range(args.warmup):
            x, _ = oc.thetaStep(x, dt=args.dt, theta=1.0, precision=prec)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sts = []
        for _ in range(args.steps):
            x, s = oc.thetaStep(x, dt=args.dt, theta=1.0, precision=prec)
            sts.append(s)
        wall = time.perf_counter() - t0
        out[label] = {"time_steps_per_s": args.steps / wall, "wall_s": wall,
                      "converged_steps": sum(s["converged"] for s in sts),
                      "newton_iters": sum(s["newton_iters"] for s in sts),
                      "krylov_iters": sum(s["krylov_iters"] for s in sts),
                      "factorizations": sum(s["factorizations"] for s in sts),
                      "factor_ms": sum(s["time_factor_ms"] for s in sts),
                      "solve_ms": sum(s["time_solve_ms"] for s in sts),
                      "last_norm_G": sts[-1]["norm_G"] if sts else None}
    if out["fp64"]["wall_s"] > 0:
        out["speedup_vs_fp64_gpu"] = out["mixed"]["time_steps_per_s"] / out["fp64"]["time_steps_per_s"]
    print(json.dumps(out), flush=True)


def run_newton_large(args):
    """Newton iterations on the 1-degree 360x160x20 ocean (6.9 M unknowns):
    iteration 0 with every kernel timed (per-class device time and HBM rate),
    then `--large-steps` untimed iterations (F, J, mixed solve to 1e-8,
    update) through the public host-buffer API. The FP64 path is sized and
    reported: its factor store alone exceeds the device memory."""
    import torch
    from iemic import Ocean
    from iemic import workloads as W
    torch.cuda.init()
    cfg = W.global_360x160x20()
    lm = W.seeded_global_mask(cfg, 0, min_depth_frac=0.1)
    oc = Ocean(cfg, lm, forcing=None, starting_parameters=W.STARTING_PARAMETERS)
    if args.subst_threshold is not None:
        oc.setSubstitutionThreshold(args.subst_threshold)
    oc.setPar("Combined Forcing", args.setup_comb)
    x = W.rest_state_with_ts_noise(cfg, 0)
    info = oc.solverInfo()
    free, total = torch.cuda.mem_get_info()
    out = {"mode": "newton_large", "workload": "global_360x160x20", "unknowns": oc.ndim, "solver": info,
           "subst_threshold": args.subst_threshold,
           "device_memory_gb": total / 1e9}
    peaks = load_peaks()
    hbm = peaks.get("hbm_gbs", 6800.0)
    simt = 2 * 128 * 152 * peaks.get("sm_max_mhz", 2070.0) * 1e6 / 1e12
    steps = []
    f0 = None
    for it in range(args.large_steps + 1):
        timed = it == 0
        oc.kernelTiming(timed)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        F = oc.computeRHS(x)
        oc.computeJacobian(x)
        dx, st = oc.solve(-F, precision=1)
        x += dx
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        fn = float(np.linalg.norm(F))
        f0 = fn if f0 is None else f0
        steps.append({"iter": it, "timed_kernels": timed, "wall_s": wall, "norm_F": fn, "gmres_iters": st["iters"],
                      "relres": st["relres"], "factor_ms": st["time_factor_ms"], "solve_ms": st["time_solve_ms"],
                      "status": st["status"]})
        if timed:
            ks = oc.kernelStats()
            kern = {}
            for k, v in ks.items():
                if not v["launches"]:
                    continue
                e = {"ms": round(v["ms"], 3), "launches": v["launches"]}
                if v["bytes"] > 0 and v["ms"] > 0 and k != "factor_gemm":
                    e["gb_s"] = v["bytes"] / (v["ms"] * 1e-3) / 1e9
                    e["hbm_frac"] = e["gb_s"] / hbm
                if k == "factor_gemm" and v["ms"] > 0:
                    e["tflop_s"] = v["flops"] / (v["ms"] * 1e-3) / 1e12
                    e["simt_frac"] = e["tflop_s"] / simt
                kern[k] = e
            out["kernels_iter0"] = kern
            out["timing_failures"] = oc.kernelTimingFailures()
        oc.kernelTiming(False)
        print(json.dumps(steps[-1]), flush=True)
    run = steps[1:]
    out["mixed"] = {"steps": steps, "timed_iterations": len(run),
                    "newton_steps_per_s": len(run) / sum(r["wall_s"] for r in run) if run else None,
                    "norm_F_first_last": [steps[0]["norm_F"], steps[-1]["norm_F"]]}
    need64 = 8.0 * (info["factor_entries"] + info["work_entries"] + info["contrib_entries"])
    out["fp64"] = {"unavailable": "FP64 factor store + working area + contribution ring need %.0f GB of the "
                                  "device's %.0f GB" % (need64 / 1e9, total / 1e9),
                   "factor_flops": info["factor_flops"]}
    free_end, _ = torch.cuda.mem_get_info()
    out["device_used_gb"] = (total - free_end) / 1e9
    print(json.dumps(out), flush=True)


def main():
    args = parse()
    if args.mode == "newton_large":
        run_newton_large(args)
        return
    if args.mode == "newton1":
        run_newton1(args)
        return
    if args.mode == "transient":
        run_transient(args)
        return
    rank, world = dist_init()
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_ours(args, rank, world)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
