"""The incomplete-factorisation claim behind the preconditioner choice, on the
oracle's Jacobian of the 16x16x4 box (gauge pins removed): zero-fill ILU
(scipy's SuperLU ILUTP with drop tolerance 0 and fill factor 1) meets an
exactly zero pivot in natural order and after the (u, v, p, w, T, S) cell
reordering, while the complete LU is an exact solve. oracle/ilu_study.py
prints the full table (ILUT variants, the larger cases)."""
import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from helpers import box_case, make_oracle, seeded_state


@pytest.fixture(scope="module")
def box_matrix():
    from oracle.gauge import gauge_pins
    cfg, lm, frc = box_case()
    o = make_oracle(cfg, lm, frc)
    rp, ci = o.graph()
    vals, _ = o.jacobian(seeded_state(cfg, 0, uvw=0.01))
    n = o.ndim
    J = sp.csr_matrix((vals, ci, rp), shape=(n, n))
    J.eliminate_zeros()
    pins = gauge_pins(o.landm(), cfg["n"], cfg["m"], cfg["l"], cfg["periodic"])
    keep = np.setdiff1d(np.arange(n), pins)
    return J[keep][:, keep].tocsc(), keep


def test_zero_fill_ilu_meets_a_zero_pivot(box_matrix):
    A, keep = box_matrix
    order = np.array([0, 1, 3, 2, 4, 5])
    perm = np.argsort((keep // 6) * 6 + order[keep % 6], kind="stable")
    for M in (A, A[perm][:, perm].tocsc()):
        with pytest.raises(RuntimeError):
            spla.spilu(M, drop_tol=0.0, fill_factor=1, permc_spec="NATURAL", diag_pivot_thresh=0.0)


def test_complete_lu_is_exact(box_matrix):
    A, _ = box_matrix
    b = A @ np.random.default_rng(0).normal(size=A.shape[0])
    x = spla.splu(A).solve(b)
    assert np.linalg.norm(A @ x - b) <= 1e-12 * np.linalg.norm(b)
