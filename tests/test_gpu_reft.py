"""Vertical mixing on the GPU, and the GPU pinned to a state the reference
itself produced.

1. Assembly with Mixing = 2 (src/ocean/mix_imp.f: vmix_control, vmix_fun,
   the forward-difference vmix_jac) on the reference's 16x16x16 gateway basin:
   F and J bit-exact against the oracle, through the adaptive partition's
   states (T = S = 0, then both fields on).
2. The reference's regression test src/tests/reft_ocean.C on the GPU engine:
   continuation in Combined Forcing from rest to 0.02
   (test/ocean/reft_continuation_params.xml) on both solver paths, compared
   with test/ocean/ocean_reference.h5 (stored in tests/golden/): the 2-norms of
   u, v, T and S to the reference's own tolerance 1e-3, and, tighter, to 1e-7
   relative; the final Combined Forcing to 1e-9.
"""
import numpy as np
import pytest

from helpers import gateway_case, gateway_golden, make_gpu, make_oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pair():
    from iemic import workloads as W
    cfg, lm, _ = gateway_case(2)
    o = make_oracle(cfg, lm, None, W.GATEWAY_STARTING_PARAMETERS)
    g = make_gpu(cfg, lm, None, W.GATEWAY_STARTING_PARAMETERS)
    return cfg, o, g


def test_parameters_match_the_reference(pair):
    cfg, o, g = pair
    _, pars = gateway_golden()
    assert g.getPar("P_VC") == pars["P_VC"] == o.get_par("P_VC")
    assert np.array_equal(g.getLandMask(), o.landm())


def test_mixing_assembly_bit_exact_through_the_partition_states(pair):
    cfg, o, g = pair
    ref, pars = gateway_golden()
    o.set_par("COMB", pars["Combined Forcing"])
    g.setPar("Combined Forcing", pars["Combined Forcing"])
    rng = np.random.default_rng(11)
    noisy = ref.copy()
    noisy[4::6] += rng.normal(0.0, 0.5, g.ndim // 6)   # unstable stratification: convective adjustment on
    states = [np.zeros(g.ndim), ref, noisy, np.zeros(g.ndim), noisy]
    for x in states:
        Fo, Fg = o.rhs(x), g.computeRHS(x)
        assert np.array_equal(Fg, Fo), "F: %d entries differ" % int(np.sum(Fg != Fo))
        vo, excl = o.jacobian(x)
        assert excl == 0
        g.computeJacobian(x)
        vg = g.getJacobian()[2]
        assert np.array_equal(vg, vo), "J: %d entries differ" % int(np.sum(vg != vo))


def test_mixing_changes_the_residual(pair):
    """The mixing term is really there: F differs from the Mixing = 0 model on
    an unstably stratified state, in T and S rows only."""
    from iemic import workloads as W
    cfg, o, g = pair
    ref, pars = gateway_golden()
    cfg0, lm, _ = gateway_case(0)
    g0 = make_gpu(cfg0, lm, None, W.GATEWAY_STARTING_PARAMETERS)
    g0.setPar("P_VC", g.getPar("P_VC"))
    g.setPar("Combined Forcing", pars["Combined Forcing"])
    g0.setPar("Combined Forcing", pars["Combined Forcing"])
    x = ref.copy()
    x[4::6] += np.random.default_rng(3).normal(0.0, 0.5, g.ndim // 6)
    d = g.computeRHS(x) - g0.computeRHS(x)
    assert np.linalg.norm(d[4::6]) > 0 and np.linalg.norm(d[5::6]) > 0
    for t in (0, 1, 2, 3):
        assert np.all(d[t::6] == 0.0)


def test_neutral_physics_is_rejected(pair):
    cfg, o, g = pair
    from iemic.ocean import IemicError
    g.setPar("MIXP", 0.5)
    with pytest.raises(IemicError):
        g.computeRHS(np.zeros(g.ndim))
    g.setPar("MIXP", 0.0)
    g.computeRHS(np.zeros(g.ndim))


@pytest.mark.parametrize("prec", [0, 1])
def test_reft_continuation_reproduces_the_reference_state(prec):
    from iemic import workloads as W
    ref, pars = gateway_golden()
    cfg, lm, _ = gateway_case(2)
    g = make_gpu(cfg, lm, None, W.GATEWAY_STARTING_PARAMETERS)
    x, st = g.continuation(np.zeros(g.ndim), par="Combined Forcing", precision=prec, tangent="S",
                           **W.GATEWAY_CONTINUATION)
    assert st["status"] == 0 and st["reached_destination"] == 1 and st["failed_steps"] == 0, st
    assert st["par"] == pytest.approx(pars["Combined Forcing"], abs=1e-9)
    for t, name in ((0, "u"), (1, "v"), (4, "T"), (5, "S")):
        got, want = np.linalg.norm(x[t::6]), np.linalg.norm(ref[t::6])
        assert abs(got - want) < 1e-3, (name, got, want)           # src/tests/reft_ocean.C:86
        assert abs(got - want) <= 1e-7 * want, (name, got, want)
    for t in (0, 1, 2, 4, 5):
        assert np.max(np.abs(x[t::6] - ref[t::6])) <= 1e-6 * np.max(np.abs(ref[t::6]))
