"""The oracle's restatement of the theta method (ThetaModel.H + transient
Newton.H), on the CPU: a steady state is a fixed point of a time step (the
F terms vanish and B (x_old - x) forces x = x_old), and a step from a
non-steady state converges quadratically with G(x_new) at round-off."""
import numpy as np
import pytest

from helpers import box_case, make_oracle, seeded_state


def _box():
    from oracle.gauge import gauge_pins
    cfg, lm, frc = box_case()
    o = make_oracle(cfg, lm, frc)
    pins = gauge_pins(o.landm(), cfg["n"], cfg["m"], cfg["l"], cfg["periodic"])
    return cfg, o, pins


def test_steady_state_is_a_fixed_point():
    from oracle.continuation import OracleModel, newton
    from oracle.transient import theta_step
    cfg, o, pins = _box()
    o.set_par("COMB", 0.1)
    M = OracleModel(o, pins)
    xs, its, res, ok = newton(M, np.zeros(o.ndim), max_iters=20, tol=1e-10)
    assert ok, (its, res)
    for theta in (1.0, 0.5):
        xn, st = theta_step(o, xs, 0.05, theta, pins=pins)
        assert st["converged"] == 1 and st["newton_iters"] <= 2, st
        assert np.linalg.norm(xn - xs) <= 1e-8 * np.linalg.norm(xs)


@pytest.mark.parametrize("theta", [1.0, 0.5])
def test_step_converges_quadratically(theta):
    from oracle.transient import theta_step
    cfg, o, pins = _box()
    x = seeded_state(cfg, 0)
    xn, st = theta_step(o, x, 1e-2, theta, pins=pins)
    assert st["converged"] == 1 and st["newton_iters"] <= 6, st
    assert st["norm_G"] < 1e-12 and np.all(xn[pins] == x[pins])


def test_bad_arguments():
    from oracle.transient import theta_step
    cfg, o, pins = _box()
    with pytest.raises(ValueError):
        theta_step(o, np.zeros(o.ndim), 1e-2, 0.0, pins=pins)
