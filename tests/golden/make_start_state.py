"""Regenerate tests/golden/start_global96.npz (run from the repository root).

The starting point of the timed continuation of the 96x38x12 global ocean
(bench.py, workload global_96x38x12), computed on the CPU with the oracle:
the steady state at Combined Forcing 0.1 reached from rest by continuation
(step 0.05, at most 0.1), then ``--warmup`` (default 5) pseudo-arclength steps
in Salinity Forcing with the bench's options. Every solve is an exact FP64
multifrontal LU solve (oracle.multifrontal). The file holds the state, the
Salinity Forcing reached, ||F(0)||_2 and the warm-up step count. bench.py's
``--impl reference`` arm starts its CPU continuation from it, so that the CPU
and GPU arms time the same continuation from the same point.
"""
import argparse
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
HERE = os.path.dirname(os.path.abspath(__file__))
sys.path[:0] = [ROOT, os.path.join(ROOT, "i-emic_gb300")]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--out", default=os.path.join(HERE, "start_global96.npz"))
    args = ap.parse_args()
    import oracle
    from oracle.continuation import Continuation, MultifrontalModel
    from oracle.multifrontal import Plan
    from iemic import workloads as W
    cfg = W.global_96x38x12()
    lm = W.seeded_global_mask(cfg, 0)
    o = oracle.Oracle(cfg, lm)
    for name, v in W.STARTING_PARAMETERS:
        o.set_par({"Combined Forcing": "COMB", "Temperature Forcing": "TEMP", "Salinity Forcing": "SALT",
                   "Wind Forcing": "WIND"}[name], v)
    nd = o.ndim
    fscale = float(np.linalg.norm(o.rhs(np.zeros(nd))))     # ||F(0)|| at the starting parameters
    o.set_par("COMB", 0.0)
    plan = Plan(o.landm(), cfg["n"], cfg["m"], cfg["l"], cfg["periodic"])
    M = MultifrontalModel(o, plan, policy="each")
    t0 = time.time()
    C = Continuation(M, np.zeros(nd), par="COMB", ds=0.05, ds_max=0.1, destination=0.1, max_steps=20,
                     newton_tol=1e-8 * fscale, residual_test="R", predictor_bound=1e30)
    st = C.run()
    print("setup", st, "%.0f s" % (time.time() - t0), flush=True)
    assert st["reached_destination"] == 1
    C2 = Continuation(M, C.x, par="SALT", ds=0.01, ds_min=1e-8, ds_max=0.1, destination=10.0,
                      max_steps=args.warmup, max_newton=15, min_newton=1, opt_newton=3.5,
                      newton_tol=1e-8 * fscale, residual_test="R", normalize="N", tangent="S",
                      newton_chord=True, epsilon=1e-5, predictor_bound=3000.0, tan_scaling=1.0)
    st2 = C2.run()
    print("warmup", st2, "%.0f s" % (time.time() - t0), flush=True)
    np.savez_compressed(args.out, x=C2.x, salinity_forcing=np.array(C2.par), fscale=np.array(fscale),
                        warmup=np.array(args.warmup), combined_forcing=np.array(o.get_par("COMB")))


if __name__ == "__main__":
    main()
