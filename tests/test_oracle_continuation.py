"""The continuation/Newton oracle on its own (CPU): the restated drivers of
src/continuation/Continuation.H and src/newton/Newton.H converge on the
16x16x4 box and stay on the branch F(x, par) = 0."""
import numpy as np
import pytest

from helpers import box_case, make_oracle


def _box_model():
    from oracle.continuation import OracleModel
    cfg, lm, frc = box_case()
    o = make_oracle(cfg, lm, frc)
    n, m, l = cfg["n"], cfg["m"], cfg["l"]
    # gauge: two horizontally adjacent surface pressures in the north-east corner
    pins = [6 * ((n - 1) + n * (m - 1) + n * m * (l - 1)) + 3, 6 * ((n - 2) + n * (m - 1) + n * m * (l - 1)) + 3]
    return o, OracleModel(o, pins), pins


def test_gauge_solve_is_exact():
    o, M, pins = _box_model()
    rng = np.random.default_rng(5)
    x = np.zeros(o.ndim)
    x[4::6] = rng.normal(0, 0.1, o.ndim // 6)
    M.jacobian(x)
    b = M.J @ rng.normal(0, 1, o.ndim)        # a consistent right-hand side
    sol = M.solve(b)
    assert np.all(sol[pins] == 0.0)
    assert np.linalg.norm(M.J @ sol - b) <= 1e-10 * np.linalg.norm(b)


def test_newton_converges_quadratically():
    from oracle.continuation import newton
    o, M, _ = _box_model()
    o.set_par("COMB", 0.05)
    x, iters, res, ok = newton(M, np.zeros(o.ndim), max_iters=10, tol=1e-9)
    assert ok and iters <= 6, (iters, res)
    assert np.linalg.norm(o.rhs(x)) < 1e-9


@pytest.mark.parametrize("opts", [dict(), dict(normalize="O", tangent="E", tan_scaling=1e-3)])
def test_continuation_steps_stay_on_branch(opts):
    from oracle.continuation import Continuation
    o, M, _ = _box_model()
    o.set_par("COMB", 0.0)
    C = Continuation(M, np.zeros(o.ndim), par="COMB", ds=0.1, ds_max=0.5, destination=1.0,
                     newton_tol=1e-8, max_steps=3, **opts)
    st = C.run()
    assert st["steps"] == 3 and len(C.history) == 3 - st["failed_steps"] >= 2
    pars = [p for p, _, _ in C.history]
    assert all(b > a for a, b in zip(pars, pars[1:])) and pars[0] > 0
    assert np.linalg.norm(o.rhs(C.x)) < 1e-9
    assert abs(o.get_par("COMB") - C.par) == 0.0
