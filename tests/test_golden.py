"""Golden fixtures (tests/golden/, made by make_golden.py): the CPU oracle
reproduces its recorded residuals and Jacobian summaries, and builds on the
reference's real-continent 96x38x12 mask."""
import hashlib
import os

import numpy as np
import pytest
import scipy.sparse as sp

from helpers import box_case, global_case, make_oracle, seeded_state

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = {"box_seed0": (box_case, 0), "glob24_seed1": (global_case, 1)}


def summary(rp, ci, vals, F):
    n = len(rp) - 1
    J = sp.csr_matrix((vals, ci, rp), shape=(n, n))
    one = np.ones(n)
    h = hashlib.sha256(np.asarray(rp, np.int32).tobytes() + np.asarray(ci, np.int32).tobytes()).hexdigest()
    return dict(F=F, J1=J @ one, JT1=J.T @ one, Jsample=np.asarray(vals)[::97], graph_sha256=h)


def check_against_golden(name, got):
    g = np.load(os.path.join(GOLDEN, "oracle_%s.npz" % name))
    assert str(g["graph_sha256"]) == got["graph_sha256"]
    for key in ("F", "J1", "JT1", "Jsample"):
        ref = g[key]
        scale = max(np.abs(ref).max(), 1e-300)
        assert np.allclose(got[key], ref, rtol=1e-12, atol=1e-12 * scale), key


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_matches_golden(name):
    case, seed = CASES[name]
    cfg, lm, frc = case()
    o = make_oracle(cfg, lm, frc)
    x = seeded_state(cfg, seed, uvw=0.01)
    rp, ci = o.graph()
    vals, _ = o.jacobian(x)
    check_against_golden(name, summary(rp, ci, vals, o.rhs(x)))


def real_mask_case():
    from iemic import workloads as W
    cfg = W.global_96x38x12()
    lm = np.load(os.path.join(GOLDEN, "mask_global_96x38x12.npy")).astype(np.int32)
    return cfg, lm.ravel(), None


def test_real_mask_oracle():
    cfg, lm, frc = real_mask_case()
    o = make_oracle(cfg, lm, frc, params=(("Combined Forcing", 0.0),))
    assert o.ndim == 6 * 96 * 38 * 12
    assert np.abs(o.rhs(np.zeros(o.ndim))).max() == 0.0          # F(0) = 0 without forcing
    rp, ci = o.graph()
    assert np.all(np.diff(rp) <= 24) and rp[-1] <= 104 * 96 * 38 * 12
