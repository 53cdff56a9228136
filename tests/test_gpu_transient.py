"""One implicit theta-method time step on the GPU (iemic_theta_step:
ThetaModel<Ocean> of src/transient/ThetaModel.H:64-140 with the transient
Newton iteration of src/transient/Newton.H:77-110) against the oracle's
restatement (oracle/transient.py, exact solves in the same pressure gauge):
the same Newton iteration counts, states agreeing to 1e-7 relative, both
precisions, theta = 1 and 1/2, single and repeated steps; a steady state is a
fixed point; invalid theta / dt are rejected."""
import numpy as np
import pytest

from helpers import box_case, global_case, make_gpu, make_oracle, seeded_state

pytestmark = pytest.mark.gpu

CASES = {"box": (box_case, 0), "glob24": (global_case, 1)}


def _pair(name):
    case, seed = CASES[name]
    cfg, lm, frc = case()
    g = make_gpu(cfg, lm, frc)
    o = make_oracle(cfg, lm, frc)
    return cfg, g, o, seeded_state(cfg, seed)


@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("theta", [1.0, 0.5])
def test_step_matches_oracle(theta, prec):
    from oracle.transient import theta_step
    cfg, g, o, x = _pair("box")
    pins = g.getGauge()
    xo, so = theta_step(o, x, 1e-2, theta, pins=pins)
    xg, sg = g.thetaStep(x, dt=1e-2, theta=theta, precision=prec)
    assert sg["status"] == 0 and sg["converged"] == 1 and so["converged"] == 1, (sg, so)
    assert abs(sg["newton_iters"] - so["newton_iters"]) <= 1, (sg, so)
    assert sg["norm_G"] < 1e-8 and sg["norm_dx"] < 1e-8
    assert np.linalg.norm(xg - xo) <= 1e-7 * np.linalg.norm(xo), np.linalg.norm(xg - xo) / np.linalg.norm(xo)
    assert np.array_equal(xg[pins], x[pins])   # the gauge unknowns keep their values


def test_repeated_steps_match_oracle():
    from oracle.transient import theta_step
    cfg, g, o, x = _pair("glob24")
    pins = g.getGauge()
    xo, xg = x.copy(), x.copy()
    for _ in range(3):
        xo, so = theta_step(o, xo, 1e-2, 1.0, pins=pins)
        xg, sg = g.thetaStep(xg, dt=1e-2, theta=1.0, precision=1)
        assert sg["converged"] == 1 and so["converged"] == 1, (sg, so)
        assert np.linalg.norm(xg - xo) <= 1e-7 * np.linalg.norm(xo)


def test_steady_state_is_a_fixed_point():
    from oracle.continuation import OracleModel, newton
    cfg, g, o, _ = _pair("box")
    pins = g.getGauge()
    o.set_par("COMB", 0.1)
    g.setPar("Combined Forcing", 0.1)
    xs, its, res, ok = newton(OracleModel(o, pins), np.zeros(o.ndim), max_iters=20, tol=1e-10)
    assert ok
    xg, sg = g.thetaStep(xs, dt=0.05, theta=1.0, precision=1)
    assert sg["converged"] == 1 and sg["newton_iters"] <= 2, sg
    assert np.linalg.norm(xg - xs) <= 1e-8 * np.linalg.norm(xs)


def test_bad_arguments():
    from iemic import IemicError
    cfg, g, o, x = _pair("box")
    for kw in (dict(theta=0.0), dict(theta=1.5), dict(dt=0.0), dict(dt=-1e-2)):
        with pytest.raises(IemicError):
            g.thetaStep(x, **{**dict(dt=1e-2, theta=1.0), **kw})


@pytest.mark.parametrize("prec", [0, 1])
def test_step_with_integral_condition_matches_oracle(prec):
    """SRES = 0 (the reference's unit-test ocean, Mixing 1): the dense
    integral-condition row has no mass, so J2 keeps it as in J."""
    from iemic import workloads as W
    from helpers import natl8_case
    from oracle.transient import theta_step
    cfg, lm, _ = natl8_case()
    g = make_gpu(cfg, lm, None, W.NATL8_STARTING_PARAMETERS)
    o = make_oracle(cfg, lm, None, W.NATL8_STARTING_PARAMETERS)
    o.set_par("COMB", 0.5)
    g.setPar("Combined Forcing", 0.5)
    x = seeded_state(cfg, 2)
    pins = g.getGauge()
    xo, so = theta_step(o, x, 1e-2, 1.0, pins=pins)
    xg, sg = g.thetaStep(x, dt=1e-2, theta=1.0, precision=prec)
    assert sg["converged"] == 1 and so["converged"] == 1, (sg, so)
    assert abs(sg["newton_iters"] - so["newton_iters"]) <= 1, (sg, so)
    assert np.linalg.norm(xg - xo) <= 1e-7 * np.linalg.norm(xo), np.linalg.norm(xg - xo) / np.linalg.norm(xo)
