"""Adjoint of the steady state on the GPU.

- J^T lambda = b with the forward solve's factorisation (M^{-T}) against the
  oracle's exact transposed solve in the same gauge (zero at the pins).
- psi_M (Ocean::getPsiM) against the oracle's compute_psim restatement.
- d(max psi_M)/d(emip) and d(max psi_M)/d(par) by one adjoint solve against
  central finite differences of re-converged steady states (1e-5 relative),
  and through the torch.autograd wrapper.
"""
import ctypes

import numpy as np
import pytest

from helpers import box_case, global_case, make_gpu, make_oracle, seeded_state

pytestmark = pytest.mark.gpu

CASES = {"box": box_case, "glob24": global_case}
SCALE = 6.37e6 * 0.1 * 1e-6   # r0dim * udim * 1e-6 (times hdim)


def _dev(a):
    import torch
    return torch.tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda")


@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("name", sorted(CASES))
def test_transposed_solve_matches_oracle(name, prec):
    from oracle.continuation import OracleModel
    cfg, lm, frc = CASES[name]()
    g = make_gpu(cfg, lm, frc)
    o = make_oracle(cfg, lm, frc)
    x = seeded_state(cfg, 2, uvw=0.01)
    g.computeJacobian(x)
    pins = g.getGauge()
    M = OracleModel(o, pins)
    M.jacobian(x)
    rng = np.random.default_rng(11)
    b = M.J.T @ rng.normal(0, 1, g.ndim)          # consistent: orthogonal to null(J)
    lam, st = g.solve(b, precision=prec, transpose=1)
    assert st["status"] == 0, st
    relres = np.linalg.norm(M.J.T @ lam - b) / np.linalg.norm(b)
    assert relres <= 1e-8 and st["relres"] <= 1e-8, (relres, st)
    assert np.all(lam[pins] == 0.0)
    keep = M.keep
    import scipy.sparse.linalg as spla
    ref = np.zeros(g.ndim)
    ref[keep] = spla.spsolve(M.J[keep][:, keep].T.tocsc(), b[keep])
    assert np.linalg.norm(lam - ref) / np.linalg.norm(ref) <= 1e-5


def _steady_box(comb=0.05):
    cfg, lm, frc = box_case()
    g = make_gpu(cfg, lm, frc)
    g.setPar("Combined Forcing", comb)
    x, st = g.newton(np.zeros(g.ndim), precision=0, max_iters=20, tol=1e-10)
    assert st["status"] == 0, st
    return cfg, lm, frc, g, x


def test_psim_matches_oracle():
    cfg, lm, frc, g, x = _steady_box()
    o = make_oracle(cfg, lm, frc)
    o.set_par("COMB", 0.05)
    psi, lo, hi = g.getPsiM(x)
    ref = o.psim(x).reshape(cfg["l"] + 1, cfg["m"] + 1) * SCALE * cfg["hdim"]
    assert np.allclose(psi, ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max())
    assert hi == pytest.approx(ref.max(), rel=1e-12) and hi > 0
    assert lo == pytest.approx(ref.min(), rel=1e-12, abs=1e-14)


def _g_at(g, x0, name=None, field=None, par=None, value=None):
    if field is not None:
        g.setForcing(**{name: field.ravel()})
    if par is not None:
        g.setPar(par, value)
    x, st = g.newton(x0, precision=0, max_iters=20, tol=1e-10)
    assert st["status"] == 0, st
    return g.getPsiM(x)[2]


@pytest.mark.parametrize("prec", [0, 1])
def test_adjoint_gradient_matches_finite_differences(prec):
    cfg, lm, frc, g, x = _steady_box()
    gval, fields, pars, st = g.adjointPsiM(x, pars=("Salinity Forcing", "Wind Forcing"), precision=prec)
    assert st["status"] == 0 and st["relres"] <= 1e-10, st
    assert gval == pytest.approx(g.getPsiM(x)[2], rel=1e-13)
    ge = fields["emip"]
    emip0 = np.asarray(frc["emip"], dtype=np.float64).reshape(cfg["m"], cfg["n"])
    # the three largest emip sensitivities
    cells = np.dstack(np.unravel_index(np.argsort(-np.abs(ge).ravel())[:3], ge.shape))[0]
    h = 1e-4
    for j, i in cells:
        fp, fm = emip0.copy(), emip0.copy()
        fp[j, i] += h
        fm[j, i] -= h
        gp = _g_at(g, x, "emip", fp)
        gm = _g_at(g, x, "emip", fm)
        g.setForcing(emip=emip0.ravel())
        fd = (gp - gm) / (2 * h)
        assert abs(fd - ge[j, i]) <= 1e-5 * np.abs(ge).max(), (j, i, fd, ge[j, i])
    for par, gpar in pars.items():
        p0 = g.getPar(par)
        hp = 1e-5 * max(1.0, abs(p0))
        gp = _g_at(g, x, par=par, value=p0 + hp)
        gm = _g_at(g, x, par=par, value=p0 - hp)
        g.setPar(par, p0)
        fd = (gp - gm) / (2 * hp)
        assert abs(fd - gpar) <= 1e-5 * max(abs(gpar), abs(fd)), (par, fd, gpar)


def test_autograd_wrapper():
    import torch
    from iemic.autograd import SteadyPsiMax
    cfg, lm, frc, g, x = _steady_box()
    emip0 = np.asarray(frc["emip"], dtype=np.float64).reshape(cfg["m"], cfg["n"])
    f = torch.tensor(emip0, dtype=torch.float64, requires_grad=True)
    out = SteadyPsiMax.apply(f, g, "emip", x)
    (grad,) = torch.autograd.grad(out, f)
    _, fields, _, _ = g.adjointPsiM(x)
    assert out.item() == pytest.approx(g.getPsiM(x)[2], rel=1e-9)
    assert np.allclose(grad.numpy(), fields["emip"], rtol=1e-6, atol=1e-9 * np.abs(fields["emip"]).max())


def test_adjoint_bad_arguments():
    from iemic import IemicError
    cfg, lm, frc, g, x = _steady_box()
    with pytest.raises(IemicError):
        g.adjointPsiM(x, sector=(5, 2))
    with pytest.raises(IemicError):
        g.adjointPsiM(x, pars=(99,))


def _sector_g(g, x, sector):
    """max psi_M over the sector [i0, i1) through iemic_psim_max_grad_dev."""
    import torch
    xd = _dev(x)
    grad = torch.zeros(g.ndim, dtype=torch.float64, device="cuda")
    gv = ctypes.c_double()
    jk = (ctypes.c_int * 2)()
    rc = g.L.iemic_psim_max_grad_dev(g.handle, ctypes.c_void_p(xd.data_ptr()), sector[0], sector[1],
                                     ctypes.byref(gv), jk, ctypes.c_void_p(grad.data_ptr()))
    assert rc == 0
    return gv.value


def test_adjoint_global_sector_20_cells():
    """Gradient of the sector-restricted max overturning of a periodic global
    ocean (24x12x6, seeded land) w.r.t. the injected surface freshwater flux,
    checked by central differences on 20 seeded cells."""
    from iemic import workloads as W
    cfg, lm, _ = global_case()
    cfg = dict(cfg, its=2, ite=2)            # injected T/S forcing fields
    n, m = cfg["n"], cfg["m"]
    lat = np.linspace(-1, 1, m)[:, None] * np.ones((1, n))
    frc = dict(tatm=np.cos(np.pi * lat / 2).ravel(), emip=(0.5 * np.sin(np.pi * lat)).ravel())
    g = make_gpu(cfg, lm, frc)
    g.setPar("Combined Forcing", 0.05)
    x, st = g.newton(np.zeros(g.ndim), precision=0, max_iters=25, tol=1e-10)
    assert st["status"] == 0, st
    sector = (6, 18)
    gval, fields, _, ast = g.adjointPsiM(x, sector=sector, precision=1)
    assert ast["status"] == 0
    assert gval == pytest.approx(_sector_g(g, x, sector), rel=1e-13)
    ge = fields["emip"]
    emip0 = frc["emip"].reshape(m, n)
    landm = g.getLandMask().reshape(cfg["l"] + 2, m + 2, n + 2)
    ocean = np.argwhere(landm[cfg["l"], 1:m + 1, 1:n + 1] == 0)
    cells = ocean[np.random.default_rng(20).choice(len(ocean), 20, replace=False)]
    h = 1e-4
    scale = np.abs(ge).max()
    assert scale > 0
    for j, i in cells:
        vals = []
        for sgn in (1, -1):
            f = emip0.copy()
            f[j, i] += sgn * h
            g.setForcing(emip=f.ravel())
            xs, st = g.newton(x, precision=0, max_iters=20, tol=1e-10)
            assert st["status"] == 0, st
            vals.append(_sector_g(g, xs, sector))
        g.setForcing(emip=emip0.ravel())
        fd = (vals[0] - vals[1]) / (2 * h)
        assert abs(fd - ge[j, i]) <= 1e-5 * scale, (j, i, fd, ge[j, i], scale)
