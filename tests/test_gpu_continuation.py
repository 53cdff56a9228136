"""GPU Newton and pseudo-arclength continuation against the oracle drivers.

Both sides run the same restated algorithms (src/newton/Newton.H,
src/continuation/Continuation.H) from the same state and parameters; the
oracle solves exactly in the GPU solver's gauge, the GPU to a relative
residual of 1e-8. The converged points must agree: the parameter to 1e-7
and the state to 1e-6 (relative 2-norm).
"""
import numpy as np
import pytest

from helpers import box_case, make_gpu, make_oracle

pytestmark = pytest.mark.gpu


def _pair():
    from oracle.continuation import OracleModel
    cfg, lm, frc = box_case()
    g = make_gpu(cfg, lm, frc)
    o = make_oracle(cfg, lm, frc)
    g.computeJacobian(np.zeros(g.ndim))
    M = OracleModel(o, g.getGauge())
    return g, o, M


@pytest.mark.parametrize("prec", [0, 1])
def test_newton_matches_oracle(prec):
    from oracle.continuation import newton
    g, o, M = _pair()
    g.setPar("Combined Forcing", 0.05)
    o.set_par("COMB", 0.05)
    x0 = np.zeros(g.ndim)
    xr, it_r, res_r, ok_r = newton(M, x0, max_iters=10, tol=1e-9)
    xg, st = g.newton(x0, precision=prec, max_iters=10, tol=1e-9)
    assert ok_r and st["status"] == 0, st
    assert st["iters"] == it_r
    assert st["rhs_norm"] < 1e-9
    assert np.linalg.norm(xg - xr) / np.linalg.norm(xr) <= 1e-6


@pytest.mark.parametrize("prec,opts", [
    (0, dict()),
    (1, dict()),
    (0, dict(normalize="O", tangent="E", tan_scaling=1e-3)),
    (1, dict(residual_test="R", newton_tol=1e-8, tangent="E")),
])
def test_continuation_matches_oracle(prec, opts):
    from oracle.continuation import Continuation
    g, o, M = _pair()
    g.setPar("Combined Forcing", 0.0)
    o.set_par("COMB", 0.0)
    common = dict(ds=0.1, ds_max=0.5, destination=1.0, max_steps=4)
    common.update(opts)
    common.setdefault("newton_tol", 1e-8)
    C = Continuation(M, np.zeros(g.ndim), par="COMB", **common)
    ref = C.run()
    xg, st = g.continuation(np.zeros(g.ndim), par="Combined Forcing", precision=prec, **common)
    assert st["status"] == 0, st
    for k in ("steps", "failed_steps", "newton_iters", "reached_destination"):
        assert st[k] == ref[k], (k, st, ref)
    assert abs(st["par"] - ref["par"]) <= 1e-7 * max(1.0, abs(ref["par"])), (st["par"], ref["par"])
    assert g.getPar("Combined Forcing") == st["par"]
    assert np.linalg.norm(xg - C.x) / np.linalg.norm(C.x) <= 1e-6
    assert np.linalg.norm(g.computeRHS(xg)) < 1e-6


def test_continuation_reaches_destination():
    """Secant detection lands on the destination (Continuation::detect)."""
    g, o, M = _pair()
    g.setPar("Combined Forcing", 0.0)
    xg, st = g.continuation(np.zeros(g.ndim), par="Combined Forcing", precision=1, ds=0.02, ds_max=0.05,
                            destination=0.1, max_steps=40, newton_tol=1e-8)
    assert st["reached_destination"] == 1, st
    assert abs(st["par"] - 0.1) < 1e-7
    assert np.linalg.norm(g.computeRHS(xg)) < 1e-6


def test_bad_continuation_options():
    from iemic import IemicError
    g, o, M = _pair()
    with pytest.raises(IemicError):
        g.continuation(np.zeros(g.ndim), par="Combined Forcing", normalize="X")
    with pytest.raises(IemicError):
        g.continuation(np.zeros(g.ndim), par="Combined Forcing", epsilon=0.0)
