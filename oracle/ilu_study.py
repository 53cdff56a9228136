"""Incomplete-factorisation preconditioners on the THCM Jacobian -- TEST INFRASTRUCTURE / STUDY.

Measures, on the CPU, what an ILU-type preconditioner applied to the whole
Jacobian (the spec alternative to the nested-dissection LU the GPU
path uses) achieves on this saddle-point system: right-preconditioned
GMRES(100) to ||b - J x|| <= 1e-8 ||b|| on J x = b with b = J x_true, in the
GPU solver's pressure gauge (pinned pressures and their rows removed).

Preconditioners (scipy's SuperLU ILUTP, threshold ILU with partial pivoting):
  ilu0-nat   drop 0, fill factor 1, natural order (closest to ILU(0))
  ilu0-cell  the same after reordering each cell to (u, v, p, w, T, S)
             (a symmetric permutation: the continuity rows keep their zero
             diagonal)
  ilu0-swap  rows of each cell's continuity (p) and hydrostatic (w)
             equations exchanged, so that the diagonal holds dw/dz and dp/dz
             instead of the zero p-p and the w-w entries
  ilut-swap-1e-4  the same row exchange with drop tolerance 1e-4
  ilut-1e-3 / ilut-1e-4 / ilut-1e-5   drop tolerance, fill factor up to 20, COLAMD order
  lu         complete sparse LU (the exact solve, for scale)
Reported per case: GMRES iterations, nnz(L + U) / nnz(J) (the bytes one
application streams, relative to the matrix), factor and solve seconds.

Run: python -m oracle.ilu_study [case ...]  (cases: box, glob24, gateway)
"""
import sys
import time

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla


def _case(name):
    sys.path[:0] = ["tests", "i-emic_gb300"]
    from helpers import box_case, gateway_case, global_case, make_oracle, seeded_state
    from iemic import workloads as W
    if name == "box":
        cfg, lm, frc = box_case()
        o = make_oracle(cfg, lm, frc)
        x = seeded_state(cfg, 0, uvw=0.01)
    elif name == "glob24":
        cfg, lm, frc = global_case()
        o = make_oracle(cfg, lm, frc)
        x = seeded_state(cfg, 1, uvw=0.01)
    else:
        cfg, lm, frc = gateway_case(2)
        o = make_oracle(cfg, lm, frc, W.GATEWAY_STARTING_PARAMETERS)
        o.set_par("COMB", 0.02)
        x = seeded_state(cfg, 2, uvw=0.01)
    return cfg, o, x


def study(name, out=sys.stdout):
    from .gauge import gauge_pins
    cfg, o, x = _case(name)
    rp, ci = o.graph()
    vals, _ = o.jacobian(x)
    n = o.ndim
    J = sp.csr_matrix((vals, ci, rp), shape=(n, n))
    J.eliminate_zeros()
    pins = gauge_pins(o.landm(), cfg["n"], cfg["m"], cfg["l"], cfg["periodic"])
    keep = np.setdiff1d(np.arange(n), pins)
    A = J[keep][:, keep].tocsc()
    xt = np.random.default_rng(0).normal(size=A.shape[0])
    b = A @ xt
    # cell reordering (u, v, p, w, T, S): unknown t of a cell goes to position order[t]
    order = np.array([0, 1, 3, 2, 4, 5])
    g = keep
    cellpos = (g // 6) * 6 + order[g % 6]
    perm = np.argsort(cellpos, kind="stable")
    # row exchange p <-> w inside each cell (a left permutation)
    kpos = {gg: q for q, gg in enumerate(g)}
    swap = np.arange(A.shape[0])
    for q, gg in enumerate(g):
        t = gg % 6
        if t in (2, 3):
            other = gg + (1 if t == 2 else -1)
            if other in kpos:
                swap[q] = kpos[other]
    rows = []
    nat = dict(drop_tol=0.0, fill_factor=1, permc_spec="NATURAL", diag_pivot_thresh=0.0)
    for label, kw, p, rsw in (("ilu0-nat", dict(nat), None, False),
                              ("ilu0-cell", dict(nat), perm, False),
                              ("ilu0-swap", dict(nat), None, True),
                              ("ilut-swap-1e-4", dict(drop_tol=1e-4, fill_factor=20, permc_spec="NATURAL",
                                                      diag_pivot_thresh=0.0), None, True),
                              ("ilut-1e-3", dict(drop_tol=1e-3, fill_factor=20), None, False),
                              ("ilut-1e-4", dict(drop_tol=1e-4, fill_factor=20), None, False),
                              ("ilut-1e-5", dict(drop_tol=1e-5, fill_factor=20), None, False),
                              ("lu", None, None, False)):
        Ap = A if p is None else A[p][:, p].tocsc()
        bp = b if p is None else b[p]
        if rsw:
            Ap = A[swap].tocsc()
            bp = b[swap]
        t0 = time.perf_counter()
        try:
            F = spla.splu(Ap) if kw is None else spla.spilu(Ap, **kw)
        except RuntimeError as e:   # a zero pivot that ILUTP could not repair
            rows.append((label, None, None, None, None, str(e)[:40]))
            continue
        tf = time.perf_counter() - t0
        fill = (F.L.nnz + F.U.nnz) / Ap.nnz
        M = spla.LinearOperator(Ap.shape, matvec=F.solve, dtype=np.float64)
        AM = spla.LinearOperator(Ap.shape, matvec=lambda v: Ap @ F.solve(v), dtype=np.float64)
        count = [0]

        def cb(_):
            count[0] += 1

        t0 = time.perf_counter()
        kwg = dict(atol=0.0, restart=100, maxiter=10, callback=cb, callback_type="pr_norm")
        try:
            y, info = spla.gmres(AM, bp, rtol=1e-8, **kwg)
        except TypeError:
            y, info = spla.gmres(AM, bp, tol=1e-8, **kwg)
        ts = time.perf_counter() - t0
        xs = F.solve(y)
        rel = np.linalg.norm(Ap @ xs - bp) / np.linalg.norm(bp)
        rows.append((label, count[0], fill, tf, ts, "%.1e" % rel))
    print("case %s: %d unknowns (%d pinned), nnz(J) %d" % (name, A.shape[0], len(pins), A.nnz), file=out)
    print("%-15s %8s %10s %9s %9s %s" % ("precond", "GMRES it", "nnz(L+U)/J", "factor s", "solve s", "final relres"),
          file=out)
    for r in rows:
        if r[1] is None:
            print("%-15s %8s %10s %9s %9s %s" % (r[0], "-", "-", "-", "-", r[5]), file=out)
        else:
            print("%-15s %8d %10.2f %9.2f %9.2f %s" % r, file=out)
    out.flush()
    return rows


if __name__ == "__main__":
    for c in (sys.argv[1:] or ["box", "glob24", "gateway"]):
        study(c)
