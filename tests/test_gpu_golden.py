"""GPU assembly against the golden fixtures, and the whole Newton-step path
on the reference's real-continent 96x38x12 mask."""
import numpy as np
import pytest
import scipy.sparse as sp

from helpers import make_gpu, make_oracle, seeded_state
from test_golden import CASES, check_against_golden, real_mask_case, summary

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", sorted(CASES))
def test_gpu_matches_golden(name):
    case, seed = CASES[name]
    cfg, lm, frc = case()
    g = make_gpu(cfg, lm, frc)
    x = seeded_state(cfg, seed, uvw=0.01)
    F = g.computeRHS(x)
    g.computeJacobian(x)
    rp, ci, vals = g.getJacobian()
    check_against_golden(name, summary(rp, ci, vals, F))


def test_real_mask_assembly_and_solve():
    cfg, lm, frc = real_mask_case()
    g = make_gpu(cfg, lm, frc)
    o = make_oracle(cfg, lm, frc)
    x = seeded_state(cfg, 4, uvw=0.01)
    F = g.computeRHS(x)
    assert np.array_equal(F, o.rhs(x))
    g.computeJacobian(x)
    rp, ci, vals = g.getJacobian()
    assert np.array_equal(vals, o.jacobian(x)[0])
    J = sp.csr_matrix((vals, ci, rp), shape=(g.ndim, g.ndim))
    for prec in (1, 0):
        dx, st = g.solve(-F, precision=prec)
        assert st["status"] == 0, st
        assert np.linalg.norm(J @ dx + F) <= 1e-8 * np.linalg.norm(F)
