"""The CPU oracle checked against the reference's own known answers
(src/tests/test_ocean.C, src/tests/TestDefinitions.H)."""
import numpy as np
import pytest
import scipy.sparse as sp

import oracle
from helpers import box_case, global_case, make_oracle, seeded_state


@pytest.fixture(scope="module")
def box():
    cfg, lm, frc = box_case()
    return cfg, make_oracle(cfg, lm, frc)


def test_rhs_zero_at_rest_without_forcing():
    # test_ocean.C:42-50 (RHSNorm): ||F(0)|| < 1e-6 with zero forcing
    cfg, lm, frc = box_case()
    o = oracle.Oracle(cfg, lm)
    assert np.linalg.norm(o.rhs(np.zeros(o.ndim))) < 1e-6
    cfg, lm, _ = global_case()
    o = oracle.Oracle(cfg, lm)
    assert np.linalg.norm(o.rhs(np.zeros(o.ndim))) < 1e-6


def test_mass_matrix_values(box):
    # test_ocean.C:61-125 (MassMat): -Ro on u,v (where nonzero), 0 on w,p, -1 on T,S
    cfg, o = box
    B = o.mass()
    rosb = o.get_par("ROSB")
    for t, want in ((0, -rosb), (1, -rosb)):
        nz = B[t::6][B[t::6] != 0]
        assert np.all(nz == want)
    assert np.all(B[2::6] == 0.0) and np.all(B[3::6] == 0.0)
    assert np.all(B[4::6] == -1.0) and np.all(B[5::6] == -1.0)


def _identity_rows(o, x):
    rp, ci = o.graph()
    vals, _ = o.jacobian(x)
    ident = np.zeros(o.ndim, dtype=bool)
    for r in range(o.ndim):
        seg = vals[rp[r]:rp[r + 1]]
        cols = ci[rp[r]:rp[r + 1]]
        nz = np.nonzero(seg)[0]
        ident[r] = len(nz) == 1 and cols[nz[0]] == r and seg[nz[0]] == 1.0
    return ident


def admissible(o, x):
    """Zero the unknowns whose rows are Dirichlet identities (walls, land
    cells, surface w). The reference Jacobian treats them as fixed, so it is
    the derivative of F only on states where they vanish, as after any
    Newton step from rest."""
    x = x.copy()
    x[_identity_rows(o, x)] = 0.0
    return x


def _fd_check(o, x, ncols, seed, h=1e-6):
    # TestDefinitions.H:33-80 testEntries: |FD - J| <= max(1e-2 |J|, 1e-10) per entry.
    # Rows of land cells are skipped: the reference's rhs() multiplies them by
    # (1 - landm) = 0 (usrc.F90:580-591) while boundaries() puts identity rows
    # in J (boundary.F90:381-387), so there J is not dF/dx by construction.
    n, m, l = o.n, o.m, o.l
    lm = o.landm().reshape(l + 2, m + 2, n + 2)[1:l + 1, 1:m + 1, 1:n + 1].ravel()
    wet_rows = np.repeat(lm == 0, 6)
    rp, ci = o.graph()
    vals, excl = o.jacobian(x)
    assert excl == 0
    J = sp.csr_matrix((vals, ci, rp), shape=(o.ndim, o.ndim))
    rng = np.random.default_rng(seed)
    worst = 0.0
    active = np.nonzero(~_identity_rows(o, x))[0]
    for c in rng.choice(active, ncols, replace=False):
        e = np.zeros(o.ndim)
        e[c] = h
        fd = (o.rhs(x + e) - o.rhs(x - e)) / (2 * h)
        an = J[:, c].toarray().ravel()
        tol = np.maximum(1e-2 * np.abs(an), 1e-7)
        worst = max(worst, float(np.max((np.abs(fd - an) - tol)[wet_rows])))
    return worst


def test_fd_jacobian_box(box):
    cfg, o = box
    x = admissible(o, seeded_state(cfg, 1, uvw=0.05))
    assert _fd_check(o, x, 60, 7) <= 0.0


def test_fd_jacobian_global_with_land():
    cfg, lm, frc = global_case()
    o = make_oracle(cfg, lm, frc)
    x = admissible(o, seeded_state(cfg, 2, uvw=0.05))
    assert _fd_check(o, x, 80, 8) <= 0.0


def test_salt_conservation_columns(box):
    # test_ocean.C:242-323 (Integrals): sum_rows J(row, S col) * cos(y) dfzT over
    # S rows vanishes for interior columns -> salt is conserved by J.
    cfg, o = box
    n, m, l = cfg["n"], cfg["m"], cfg["l"]
    x = seeded_state(cfg, 3, uvw=0.02)
    rp, ci = o.graph()
    vals, _ = o.jacobian(x)
    J = sp.csr_matrix((vals, ci, rp), shape=(o.ndim, o.ndim))
    g = o.grid()
    w = np.zeros(o.ndim)
    for k in range(l):
        for j in range(m):
            w[6 * (np.arange(n) + n * j + n * m * k) + 5] = np.cos(g["y"][j + 1]) * g["dfzT"][k]
    # restoring (SRES=1, BIOT) only acts on the surface layer
    colsum = J.T @ w
    for k in range(l - 2):
        sl = [6 * (i + n * j + n * m * k) + 5 for j in range(m) for i in range(n)]
        assert np.max(np.abs(colsum[sl])) < 1e-7


def test_graph_is_sorted_and_maximal(box):
    cfg, o = box
    rp, ci = o.graph()
    lens = np.diff(rp)
    for r in range(o.ndim):
        seg = ci[rp[r]:rp[r + 1]]
        assert np.all(np.diff(seg) > 0)
    # nominal row lengths U 24, V 22, W 7, P 11, T 20, S 20 in the interior
    n, m, l = cfg["n"], cfg["m"], cfg["l"]
    cell = 5 + n * 5 + n * m * 1
    assert list(lens[6 * cell: 6 * cell + 6]) == [24, 22, 7, 11, 20, 20]


def test_fortran_csr_stays_in_domain(box):
    # fillcolA never emits a coupling to a neighbour outside the grid for valid masks
    cfg, o = box
    x = seeded_state(cfg, 4, uvw=0.05)
    o.jacobian(x)
    beg, jco, co = o.fortran_csr()
    assert np.all(np.abs(co) > 1e-10)
    assert jco.min() >= 1 and jco.max() <= o.ndim
