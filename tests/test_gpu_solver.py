"""GPU linear solves against the oracle's exact solve in the same gauge.

J x = b with b = -F(x_seeded) on the 16x16x4 box and a 24x12x6 periodic
global ocean with seeded land: the GPU returns x with the FP64 residual
||b - J x|| / ||b|| <= 1e-8 (the GMRES tolerance of Ocean::solve), zero
pressure at its gauge unknowns, and agrees with the sparse-LU solution of the
oracle's Jacobian in that gauge.
"""
import numpy as np
import pytest
import scipy.sparse as sp

from helpers import box_case, global_case, make_gpu, make_oracle, seeded_state

pytestmark = pytest.mark.gpu

CASES = {"box": box_case, "glob24": global_case}


def _setup(name, seed=0):
    from oracle.continuation import OracleModel
    cfg, lm, frc = CASES[name]()
    g = make_gpu(cfg, lm, frc)
    o = make_oracle(cfg, lm, frc)
    x = seeded_state(cfg, seed)
    F = g.computeRHS(x)
    g.computeJacobian(x)
    pins = g.getGauge()
    M = OracleModel(o, pins)
    M.jacobian(x)
    return g, o, M, x, F, pins


@pytest.mark.parametrize("name", sorted(CASES))
def test_gauge_is_surface_pressure(name):
    g, o, M, x, F, pins = _setup(name)
    n, m, l = g.n, g.m, g.l
    assert len(pins) >= 2
    for p in pins:
        assert p % 6 == 3                     # a pressure unknown
        assert (p // 6) // (n * m) == l - 1   # in the surface layer


@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("name", sorted(CASES))
def test_solve_matches_oracle(name, prec):
    g, o, M, x, F, pins = _setup(name)
    sol, st = g.solve(-F, precision=prec)
    assert st["status"] == 0, st
    J = M.J
    relres = np.linalg.norm(J @ sol + F) / np.linalg.norm(F)
    assert relres <= 1e-8 and st["relres"] <= 1e-8, (relres, st)
    assert np.all(sol[pins] == 0.0)
    ref = M.solve(-F)
    err = np.linalg.norm(sol - ref) / np.linalg.norm(ref)
    assert err <= 1e-5, err


@pytest.mark.parametrize("name", sorted(CASES))
def test_fp64_preconditioner_is_an_exact_solve(name):
    """The FP64 nested-dissection LU is a direct solver on the pinned system."""
    g, o, M, x, F, pins = _setup(name)
    g.buildPreconditioner(0)
    z = g.applyPrecon(-F, precision=0)
    ref = M.solve(-F)
    assert np.linalg.norm(z - ref) / np.linalg.norm(ref) <= 1e-6


def test_refactor_on_new_jacobian_and_reuse():
    g, o, M, x, F, pins = _setup("box")
    _, st1 = g.solve(-F, precision=1)
    _, st2 = g.solve(-F, precision=1)
    assert st1["factorizations"] == 1 and st2["factorizations"] == 0
    # a nearby state: the kept factorisation still preconditions well
    x2 = x + 1e-3 * seeded_state(g.config, 7)
    F2 = g.computeRHS(x2)
    g.computeJacobian(x2)
    sol, st3 = g.solve(-F2, precision=1, reuse_preconditioner=1)
    assert st3["factorizations"] == 0 and st3["relres"] <= 1e-8, st3
    sol, st4 = g.solve(-F2, precision=1)
    assert st4["factorizations"] == 1 and st4["relres"] <= 1e-8


def test_zero_rhs_and_bad_arguments():
    from iemic import IemicError
    g, o, M, x, F, pins = _setup("box")
    sol, st = g.solve(np.zeros(g.ndim), precision=0)
    assert np.all(sol == 0) and st["iters"] == 0
    with pytest.raises(IemicError):
        g.solve(-F, precision=7)
    with pytest.raises(IemicError):
        g.solve(-F, precision=0, restart=0)


@pytest.mark.parametrize("prec", [0, 1])
def test_kernel_timing_through_graphs(prec):
    """Timing on replays the same graphs with event nodes, every launch timed.
    Untimed solves run the GMRES cycles as device-driven graphs (Givens
    rotations and back substitution on the device), timed ones step the same
    iteration from the host: same iteration counts, solutions equal to
    rounding; two timed solves are bit-identical."""
    g, o, M, x, F, pins = _setup("glob24")
    sol0, st0 = g.solve(-F, precision=prec)
    g.kernelTiming(True)
    g.computeJacobian(x)                             # same J again: the next solve refactors
    sol1, st1 = g.solve(-F, precision=prec)          # captured with timing nodes
    assert st1["factorizations"] == 1, st1
    sol2, st2 = g.solve(-F, precision=prec, reuse_preconditioner=1)
    ks = g.kernelStats()
    tr = g.kernelTrace()
    assert g.kernelTimingFailures() == 0
    assert len(tr) == sum(k["launches"] for k in ks.values())
    g.kernelTiming(False)
    assert abs(st0["iters"] - st1["iters"]) <= 1, (st0, st1)
    assert np.linalg.norm(sol0 - sol1) <= 1e-9 * np.linalg.norm(sol1), (st0, st1)
    assert np.array_equal(sol1, sol2)
    fac = [ks[c] for c in ("factor_gemm", "factor_panel", "factor_inverse", "factor_setup")]
    assert sum(k["launches"] for k in fac) > 0 and sum(k["ms"] for k in fac) > 0, ks
    assert ks["solve_gemv"]["launches"] > 0 and ks["solve_gemv"]["ms"] > 0, ks


def test_nan_state_is_reported_not_faulted():
    """A Newton iterate that went to NaN: the factorisation's pivot search stays
    inside its blocks and the solve reports NaN/Inf instead of touching memory
    outside the fronts."""
    from iemic import IemicError
    g, o, M, x, F, pins = _setup("glob24")
    xb = x.copy()
    xb[4::6][::7] = np.nan
    g.computeJacobian(xb)
    with pytest.raises(IemicError) as ei:
        g.solve(-F, precision=1)
    assert ei.value.code == -4
    g.computeJacobian(x)                  # the handle recovers with a finite Jacobian
    sol, st = g.solve(-F, precision=1)
    assert st["status"] == 0 and st["relres"] <= 1e-8


@pytest.mark.parametrize("prec", [0, 1])
def test_block_substitution_solves(prec):
    """Substitution over inverted 256-row diagonal blocks (forced on a small
    case): forward solves match the oracle; a transposed solve then builds the
    whole inverses in place, and forward solves keep matching afterwards."""
    g, o, M, x, F, pins = _setup("glob24")
    g.setSubstitutionThreshold(0)
    sol, st = g.solve(-F, precision=prec)
    assert st["status"] == 0 and st["relres"] <= 1e-8 and st["factorizations"] == 1, st
    ref = M.solve(-F)
    assert np.linalg.norm(sol - ref) / np.linalg.norm(ref) <= 1e-5
    assert np.all(sol[pins] == 0.0)
    b = M.J.T @ np.random.default_rng(3).normal(size=g.ndim)
    lam, st = g.solve(b, precision=prec, transpose=1)
    assert st["status"] == 0 and np.linalg.norm(M.J.T @ lam - b) <= 1e-8 * np.linalg.norm(b), st
    sol2, st = g.solve(-F, precision=prec, reuse_preconditioner=1)
    assert st["factorizations"] == 0 and st["relres"] <= 1e-8, st
    assert np.linalg.norm(sol2 - ref) / np.linalg.norm(ref) <= 1e-5
    g.setSubstitutionThreshold(12288)


def test_product_sweeps_match_substitution():
    """Whole-inverse plans apply the stored products L21 Linv11 and
    Uinv11 U12 (one GEMV launch per level and sweep); the same factors applied
    by block substitution (threshold 0) give the same M^{-1} b: in FP64 to
    rounding, and in FP32 to the same accuracy against the exact solve (the
    FP32 factors' own error, which GMRES removes)."""
    g, o, M, x, F, pins = _setup("glob24")
    ref = M.solve(-F)
    out = {}
    for thr in (12288, 0):
        g.setSubstitutionThreshold(thr)
        for prec in (0, 1):
            g.buildPreconditioner(prec)
            out[thr, prec] = g.applyPrecon(-F, precision=prec)
    g.setSubstitutionThreshold(12288)
    d = np.linalg.norm(out[12288, 0] - out[0, 0]) / np.linalg.norm(out[0, 0])
    assert d <= 1e-10, d
    e_prod = np.linalg.norm(out[12288, 1] - ref) / np.linalg.norm(ref)
    e_sub = np.linalg.norm(out[0, 1] - ref) / np.linalg.norm(ref)
    assert e_prod <= 1.5 * e_sub + 1e-6, (e_prod, e_sub)   # FP32 factors: about 6e-2 both ways here


def test_elimination_tree_listing():
    """iemic_get_fronts agrees with the solver's size report: one root, parents
    on higher levels, own unknowns summing to the reduced system."""
    g, o, M, x, F, pins = _setup("glob24")
    fr = g.fronts()
    info = g.solverInfo()
    nf, nb = fr["nf"].astype(np.int64), fr["nb"].astype(np.int64)
    assert len(nf) == info["fronts"]
    assert nf.sum() == info["reduced_unknowns"]
    roots = np.nonzero(fr["parent"] < 0)[0]
    assert len(roots) == 1 and nb[roots[0]] == 0
    child = fr["parent"] >= 0
    assert np.all(fr["level"][fr["parent"][child]] > fr["level"][child])
    assert fr["level"].max() + 1 == info["levels"]
    assert (nf * nf + 2 * nf * nb).sum() == info["factor_entries"]
    assert ((nf + nb) ** 2).sum() == info["front_entries"]
