"""The integral condition on S (SRES = 0) and the fixed pressure points in
the oracle, checked against the known answers of the reference's own
src/tests/test_ocean.C on its ocean (test/ocean/ocean_params.xml: 8x8x4
mask_natl8, Mixing = 1, SRES = 0):

- F(0) = 0 with Combined Forcing 0 (RHSNorm, test_ocean.C:42-57);
- the mass matrix has a zero in the integral-condition row (MassMat,
  test_ocean.C:108-125);
- salt conservation: for every S unknown below the top two levels the
  integral-condition weights of its Jacobian column sum to zero (Integrals,
  test_ocean.C:242-300), to 1e-7;
plus the structure THCM::intcond_S and fixPressurePoints give the rows
(src/ocean/THCM.C:2180-2297) and the zero net salt flux of the forcing
(qint, src/ocean/forcing.F90:121-160)."""
import numpy as np
import pytest
import scipy.sparse as sp

from helpers import make_oracle, natl8_case, seeded_state


def _oracle(comb=0.0, **kw):
    from iemic import workloads as W
    cfg, lm, _ = natl8_case(**kw)
    o = make_oracle(cfg, lm, None, W.NATL8_STARTING_PARAMETERS)
    o.set_par("COMB", comb)
    return cfg, o


def _rowintcon(cfg):
    n, m, l = cfg["n"], cfg["m"], cfg["l"]
    return 6 * ((l - 1) * n * m + n * (m - 1) + n - 1) + 5


def test_rhs_zero_at_rest_without_forcing():
    cfg, o = _oracle(0.0)
    assert np.linalg.norm(o.rhs(np.zeros(o.ndim))) < 1e-6


def test_mass_matrix_zero_in_the_integral_row():
    cfg, o = _oracle(0.0)
    B = o.mass()
    r = _rowintcon(cfg)
    assert B[r] == 0.0
    lm = o.landm().reshape(cfg["l"] + 2, cfg["m"] + 2, cfg["n"] + 2)[1:-1, 1:-1, 1:-1].ravel()
    ocean = lm == 0
    assert np.all(B[4::6][ocean] == -1.0)
    S = B[5::6][ocean]
    assert np.all((S == -1.0) | (S == 0.0)) and np.sum(S == 0.0) == 1


def test_salt_conservation_of_the_jacobian():
    cfg, o = _oracle(0.0)
    x = np.zeros(o.ndim)
    vals, excl = o.jacobian(x)
    assert excl == 0
    rp, ci = o.graph()
    J = sp.csr_matrix((vals, ci, rp), shape=(o.ndim, o.ndim))
    r = _rowintcon(cfg)
    coef = J.getrow(r).toarray().ravel() * -1.0     # the condition's weights, sint_sign = -1
    coef[r] = 0.0                                   # test_ocean.C:266-268
    n, m, l = cfg["n"], cfg["m"], cfg["l"]
    for k in range(l - 2):
        for j in range(m):
            for i in range(n):
                c = 6 * (k * n * m + j * n + i) + 5
                col = J[:, c].toarray().ravel()
                assert abs(coef @ col) < 1e-7, (i, j, k)


def test_integral_row_structure_and_value():
    cfg, o = _oracle(1.0)
    x = seeded_state(cfg, 3, uvw=0.01)
    r = _rowintcon(cfg)
    rp, ci = o.graph()
    assert rp[r + 1] - rp[r] == cfg["n"] * cfg["m"] * cfg["l"]
    assert np.array_equal(ci[rp[r]:rp[r + 1]], np.arange(5, o.ndim, 6))
    vals, _ = o.jacobian(x)
    F = o.rhs(x)
    w = -vals[rp[r]:rp[r + 1]]
    assert F[r] == pytest.approx(-(w @ x[5::6]), rel=1e-13)
    # weights: cos(y_j) dfzT(k) on ocean cells, zero on land
    lm = o.landm().reshape(cfg["l"] + 2, cfg["m"] + 2, cfg["n"] + 2)[1:-1, 1:-1, 1:-1].ravel()
    assert np.all(w[lm != 0] == 0.0) and np.all(w[lm == 0] > 0.0)


def test_forcing_has_zero_net_salt_flux():
    cfg, o = _oracle(1.0)
    frc = o.frc()
    n, m, l = cfg["n"], cfg["m"], cfg["l"]
    y = o.grid()["y"]                               # y(0:m+1)
    lm = o.landm().reshape(l + 2, m + 2, n + 2)
    tot = 0.0
    area = 0.0
    for j in range(m):
        for i in range(n):
            wgt = np.cos(y[j + 1]) * (1 - lm[l, j + 1, i + 1])
            tot += frc[6 * ((l - 1) * n * m + j * n + i) + 5] * wgt
            area += wgt
    assert abs(tot) <= 1e-12 * area * np.max(np.abs(frc[5::6]))


def test_jacobian_matches_differences_with_the_integral_row():
    cfg, o = _oracle(1.0)
    x = seeded_state(cfg, 4, uvw=0.0)
    vals, _ = o.jacobian(x)
    rp, ci = o.graph()
    J = sp.csr_matrix((vals, ci, rp), shape=(o.ndim, o.ndim))
    lm = o.landm().reshape(cfg["l"] + 2, cfg["m"] + 2, cfg["n"] + 2)[1:-1, 1:-1, 1:-1].ravel()
    wet = lm == 0                                    # land unknowns are identity rows of J
    v = np.zeros(o.ndim)
    v[4::6] = np.random.default_rng(2).normal(size=o.ndim // 6) * wet
    v[5::6] = np.random.default_rng(3).normal(size=o.ndim // 6) * wet
    h = 1e-6
    fd = (o.rhs(x + h * v) - o.rhs(x - h * v)) / (2 * h)
    assert np.linalg.norm(J @ v - fd) <= 1e-6 * np.linalg.norm(fd)


def test_fixed_pressure_points_are_identity_rows():
    cfg, o = _oracle(1.0, fix_pressure_points=1)
    n, m, l = cfg["n"], cfg["m"], cfg["l"]
    rows = [6 * ((l - 1) * n * m + n * (m - 1) + n - 1) + 3, 6 * ((l - 1) * n * m + n * (m - 1) + n - 2) + 3]
    x = seeded_state(cfg, 5, uvw=0.01)
    vals, _ = o.jacobian(x)
    rp, ci = o.graph()
    F = o.rhs(x)
    B = o.mass()
    for r in rows:
        seg, cols = vals[rp[r]:rp[r + 1]], ci[rp[r]:rp[r + 1]]
        assert np.all(seg[cols == r] == 1.0) and np.all(seg[cols != r] == 0.0)
        assert F[r] == 0.0 and B[r] == 0.0


def test_integral_row_on_land_is_rejected():
    import oracle
    cfg, lm, _ = natl8_case()
    with pytest.raises(ValueError):
        oracle.Oracle(dict(cfg, intcon_i=0, intcon_j=0), lm)
