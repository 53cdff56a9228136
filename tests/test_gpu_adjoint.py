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
