"""The CPU oracle pinned to a state the reference itself produced.

src/tests/reft_ocean.C runs a continuation in Combined Forcing from rest to
0.02 on the 16x16x16 gateway basin with vertical mixing (Mixing = 2,
test/ocean/reft_ocean_params.xml, reft_continuation_params.xml) and compares
the 2-norms of u, v, T and S (the fields not determined up to a constant)
with test/ocean/ocean_reference.h5 to 1e-3. The restated continuation
(oracle/continuation.py) on the restated model (oracle/thcm_oracle.cpp,
mixing included) must reproduce them; without mixing it must not."""
import os

import numpy as np
import pytest

from helpers import gateway_case, gateway_golden, make_oracle

# The full continuation takes about six minutes on the CPU (a dozen exact
# sparse LU factorisations of 24,576 unknowns); it runs when IEMIC_SLOW_TESTS=1.
# The GPU suite runs the same continuation on the GPU engine against the same
# reference state (tests/test_gpu_reft.py).
slow = pytest.mark.skipif(os.environ.get("IEMIC_SLOW_TESTS", "0") in ("", "0"),
                          reason="six-minute CPU continuation; set IEMIC_SLOW_TESTS=1")


def _run(vmix):
    from iemic import workloads as W
    from oracle.continuation import Continuation, OracleModel
    from oracle.gauge import gauge_pins
    cfg, lm, _ = gateway_case(vmix)
    o = make_oracle(cfg, lm, None, W.GATEWAY_STARTING_PARAMETERS)
    M = OracleModel(o, gauge_pins(o.landm(), cfg["n"], cfg["m"], cfg["l"], cfg["periodic"]))
    opts = dict(W.GATEWAY_CONTINUATION, newton_chord=False)
    C = Continuation(M, np.zeros(o.ndim), par="COMB", tangent="S", **opts)
    st = C.run()
    return o, C, st


def test_reference_mask_and_parameters():
    """The stored land mask is the one THCM built from data/mkmask/mask_gateway
    (checked when the fixture was made), and the parameters the reference
    stored with its state match the oracle's stpnt with Mixing = 2."""
    from iemic import workloads as W
    _, pars = gateway_golden()
    cfg, lm, _ = gateway_case()
    o = make_oracle(cfg, lm, None, W.GATEWAY_STARTING_PARAMETERS)
    assert np.array_equal(o.landm().reshape(lm.shape), lm)
    for name, key in (("P_VC", "P_VC"), ("Vertical Peclet-Number", "PE_V"), ("Rossby-Number", "ROSB"),
                      ("Rayleigh-Number", "RAYL"), ("AL_T", "AL_T"), ("LAMB", "LAMB"), ("Energy", "ENER"),
                      ("ALPC", "ALPC"), ("SPL1", "SPL1"), ("MIXP", "MIXP"), ("MKAP", "MKAP")):
        assert o.get_par(key) == pytest.approx(pars[name], rel=1e-15, abs=0.0), name


def test_reference_state_is_a_root_of_the_restated_model():
    """The reference's final state solves the restated model (mixing on) to
    the accuracy of the reference's own Newton iteration (tolerance 1e-2 on
    the update); with mixing off it is far from a root."""
    from iemic import workloads as W
    ref, pars = gateway_golden()
    norms = {}
    for vmix in (2, 0):
        cfg, lm, _ = gateway_case(vmix)
        o = make_oracle(cfg, lm, None, W.GATEWAY_STARTING_PARAMETERS)
        o.set_par("COMB", pars["Combined Forcing"])
        norms[vmix] = (np.linalg.norm(o.rhs(ref)), np.linalg.norm(o.rhs(np.zeros(o.ndim))))
    assert norms[2][0] <= 1e-6 * norms[2][1], norms
    assert norms[0][0] >= 1e-3 * norms[0][1], norms


def test_mixing_jacobian_matches_differences():
    """J with mixing (the reference's forward differences of vmix_fun over a
    column partition) against central differences of F at a state with
    unstable stratification (convective adjustment active)."""
    from iemic import workloads as W
    import scipy.sparse as sp
    ref, pars = gateway_golden()
    cfg, lm, _ = gateway_case(2)
    o = make_oracle(cfg, lm, None, W.GATEWAY_STARTING_PARAMETERS)
    o.set_par("COMB", pars["Combined Forcing"])
    x = ref.copy()
    rng = np.random.default_rng(7)
    x[4::6] += rng.normal(0.0, 0.5, o.ndim // 6)     # overturn the stratification in places
    vals, outside = o.jacobian(x)
    assert outside == 0
    rp, ci = o.graph()
    J = sp.csr_matrix((vals, ci, rp), shape=(o.ndim, o.ndim))
    wet = o.landm().reshape(18, 18, 18)[1:-1, 1:-1, 1:-1].ravel() == 0
    for t in (4, 5):                                   # T and S directions
        v = np.zeros(o.ndim)
        v[t::6] = rng.normal(0.0, 1.0, o.ndim // 6) * wet
        h = 1e-6
        fd = (o.rhs(x + h * v) - o.rhs(x - h * v)) / (2 * h)
        o.jacobian(x)
        for q in (4, 5):
            a, b = (J @ v)[q::6], fd[q::6]
            assert np.linalg.norm(a - b) <= 1e-5 * np.linalg.norm(b), (t, q, np.linalg.norm(a - b), np.linalg.norm(b))


@slow
def test_continuation_reproduces_reference_state():
    ref, pars = gateway_golden()
    o, C, st = _run(2)
    assert st["reached_destination"] == 1 and st["failed_steps"] == 0
    assert C.par == pytest.approx(pars["Combined Forcing"], abs=1e-9)
    for t, name in ((0, "u"), (1, "v"), (4, "T"), (5, "S")):
        got, want = np.linalg.norm(C.x[t::6]), np.linalg.norm(ref[t::6])
        assert abs(got - want) < 1e-3, (name, got, want)          # the reference's own tolerance
        assert abs(got - want) <= 1e-7 * want, (name, got, want)  # what the restatement reaches
    # entry by entry, the fields that are unique (u, v, w, T, S) agree too
    for t in (0, 1, 2, 4, 5):
        assert np.max(np.abs(C.x[t::6] - ref[t::6])) <= 1e-6 * np.max(np.abs(ref[t::6]))


@slow
def test_golden_distinguishes_mixing():
    ref, _ = gateway_golden()
    _, C, st = _run(0)
    assert st["reached_destination"] == 1
    assert abs(np.linalg.norm(C.x[4::6]) - np.linalg.norm(ref[4::6])) > 1e-2
