"""The integral condition on S (SRES = 0) and the fixed pressure points on
the GPU, against the oracle, on the reference's unit-test ocean
(test/ocean/ocean_params.xml: 8x8x4 mask_natl8, Mixing = 1, SRES = 0) and a
24x12x6 periodic ocean with SRES = 0.

The Jacobian (its dense integral-condition row included) and the mass
matrix are bit-exact; F is bit-exact except in the integral-condition row,
a sum over all S unknowns whose order differs (1e-12 relative). Solves of
the dense-row Jacobian (the factorisation takes that row as an identity row,
the preconditioner restores it by Sherman-Morrison) reach 1e-8 and agree
with the exact solve; forward and transposed; Newton agrees with the
oracle's driver."""
import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from helpers import global_case, make_gpu, make_oracle, natl8_case, seeded_state

pytestmark = pytest.mark.gpu


def _natl8(fix=0):
    from iemic import workloads as W
    cfg, lm, _ = natl8_case(0, fix)
    return cfg, make_oracle(cfg, lm, None, W.NATL8_STARTING_PARAMETERS), make_gpu(cfg, lm, None,
                                                                                     W.NATL8_STARTING_PARAMETERS)


def _glob(fix=0):
    cfg, lm, frc = global_case()
    n, m, l = cfg["n"], cfg["m"], cfg["l"]
    surf = np.asarray(lm).reshape(l + 2, m + 2, n + 2)[l, 1:m + 1, 1:n + 1]
    j, i = np.argwhere(surf == 0)[-1]                # an ocean surface cell for the condition's row
    cfg = dict(cfg, sres=0, fix_pressure_points=fix, intcon_i=int(i), intcon_j=int(j))
    return cfg, make_oracle(cfg, lm, frc), make_gpu(cfg, lm, frc)


CASES = {"natl8": _natl8, "natl8_fixp": lambda: _natl8(1), "glob24": _glob}


def _row(cfg):
    n, m, l = cfg["n"], cfg["m"], cfg["l"]
    i = cfg.get("intcon_i", -1)
    j = cfg.get("intcon_j", -1)
    i = n - 1 if i < 0 else i
    j = m - 1 if j < 0 else j
    return 6 * ((l - 1) * n * m + n * j + i) + 5


@pytest.fixture(scope="module", params=sorted(CASES))
def trio(request):
    return CASES[request.param]()


def test_assembly_parity(trio):
    cfg, o, g = trio
    o.set_par("COMB", 0.7)
    g.setPar("Combined Forcing", 0.7)
    rp_o, ci_o = o.graph()
    rp_g, ci_g, _ = g.getJacobian(values=False)
    assert np.array_equal(rp_o, rp_g) and np.array_equal(ci_o, ci_g)
    r = _row(cfg)
    for seed in (0, 1):
        x = seeded_state(cfg, seed, uvw=0.02)
        Fo, Fg = o.rhs(x), g.computeRHS(x)
        other = np.arange(g.ndim) != r
        assert np.array_equal(Fg[other], Fo[other]), int(np.sum(Fg[other] != Fo[other]))
        assert abs(Fg[r] - Fo[r]) <= 1e-12 * max(abs(Fo[r]), 1e-300)
        vo, excl = o.jacobian(x)
        assert excl == 0
        g.computeJacobian(x)
        vg = g.getJacobian()[2]
        assert np.array_equal(vg, vo), int(np.sum(vg != vo))
    assert np.array_equal(g.getMassMat(), o.mass())


@pytest.mark.parametrize("prec", [0, 1])
def test_solve_with_the_dense_row(trio, prec):
    cfg, o, g = trio
    o.set_par("COMB", 0.7)
    g.setPar("Combined Forcing", 0.7)
    x = seeded_state(cfg, 2, uvw=0.02)
    F = g.computeRHS(x)
    g.computeJacobian(x)
    rp, ci, v = g.getJacobian()
    J = sp.csr_matrix((v, ci, rp), shape=(g.ndim, g.ndim))
    dx, st = g.solve(-F, precision=prec)
    assert st["status"] == 0, st
    assert np.linalg.norm(J @ dx + F) <= 1e-8 * np.linalg.norm(F)
    pins = g.getGauge()
    keep = np.setdiff1d(np.arange(g.ndim), pins)
    ex = np.zeros(g.ndim)
    ex[keep] = spla.splu(J[keep][:, keep].tocsc()).solve(-F[keep])
    assert np.all(dx[pins] == 0.0)
    assert np.linalg.norm(dx - ex) <= 1e-5 * np.linalg.norm(ex)
    # the transposed solve (adjoint) with the same factorisation
    bt = J.T @ np.random.default_rng(4).normal(size=g.ndim)
    lam, stt = g.solve(bt, precision=prec, transpose=1, reuse_preconditioner=1)
    assert stt["status"] == 0 and np.linalg.norm(J.T @ lam - bt) <= 1e-8 * np.linalg.norm(bt), stt


def test_newton_matches_oracle(trio):
    """Four Newton iterations from rest (no back-tracking; convergence from
    rest is slow without salinity restoring) on both sides: the iterates agree."""
    from oracle.continuation import OracleModel, newton
    cfg, o, g = trio
    o.set_par("COMB", 1e-3)
    g.setPar("Combined Forcing", 1e-3)
    g.computeJacobian(np.zeros(g.ndim))
    M = OracleModel(o, g.getGauge())
    x0 = np.zeros(g.ndim)
    xr, it_r, res_r, ok_r = newton(M, x0, max_iters=4, tol=1e-300, backtracking_steps=0)
    xg, st = g.newton(x0, precision=1, max_iters=4, tol=1e-300, backtracking_steps=0)
    assert st["iters"] == it_r == 4 and st["status"] == -3, st
    assert np.linalg.norm(xg - xr) <= 1e-6 * np.linalg.norm(xr)
    assert st["rhs_norm"] < 0.1 * st["rhs_norm0"]
