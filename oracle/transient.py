"""Implicit theta-method time step on the CPU oracle -- TEST INFRASTRUCTURE ONLY.

A numpy restatement of the reference's transient path, used as the checker of
the GPU's ``iemic_theta_step``:

- ``ThetaModel<Model>`` (src/transient/ThetaModel.H:64-140): initStep keeps
  x_old and F(x_old); computeRHS forms
      G(x) = B (x_old - x) + dt theta F(x) + dt (1 - theta) F(x_old)
  with the Epetra updates in their order (xDot = -x + x_old; Bxdot = B xDot;
  F = dt (1 - theta) F_old + dt theta F; G = Bxdot + F); computeJacobian adds
  -B / dt / theta to the diagonal; solve scales the right-hand side by
  1 / dt / theta.
- ``Newton<Model>::run`` (src/transient/Newton.H:77-110): x -= dx until
  ||dx||_inf < tol and ||G||_2 < tol; ||dx||_inf > 1e2 stops it.

Solves are exact (scipy sparse LU) in the GPU solver's pressure gauge: the
pinned pressure unknowns are held at zero and their rows dropped.
"""
import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla


def theta_step(oracle, x, dt, theta=1.0, tol=1e-8, max_newton=20, pins=()):
    """One theta step from x. Returns (x_new, stats) with stats newton_iters,
    converged, norm_G, norm_dx."""
    if not (0.0 < theta <= 1.0) or not dt > 0.0:
        raise ValueError("theta must lie in (0, 1] and dt be positive")
    o = oracle
    n = o.ndim
    rp, ci = o.graph()
    rows = np.repeat(np.arange(n), np.diff(rp))
    diag = np.full(n, -1, dtype=np.int64)
    on_diag = np.nonzero(ci == rows)[0]
    diag[rows[on_diag]] = on_diag
    keep = np.setdiff1d(np.arange(n), np.asarray(pins, dtype=np.int64))
    B = o.mass()
    a, b = dt * (1.0 - theta), dt * theta
    scale = 1.0 / dt / theta
    xold = np.array(x, dtype=np.float64)
    Fold = o.rhs(xold)

    def residual(xc):
        xdot = -xc + xold
        bxdot = B * xdot
        f = a * Fold + b * o.rhs(xc)
        return bxdot + f

    xc = xold.copy()
    G = residual(xc)
    st = dict(newton_iters=0, converged=0, norm_G=-1.0, norm_dx=0.0)
    while st["newton_iters"] < max_newton:
        vals, _ = o.jacobian(xc)
        vals = np.array(vals)
        d = diag >= 0
        vals[diag[d]] = vals[diag[d]] + (-B[d] / dt / theta)
        J2 = sp.csr_matrix((vals, ci, rp), shape=(n, n))
        rhs = G * scale
        dx = np.zeros(n)
        dx[keep] = spla.spsolve(J2[keep][:, keep].tocsc(), rhs[keep])
        st["norm_dx"] = float(np.max(np.abs(dx)))
        xc = xc - dx
        G = residual(xc)
        st["norm_G"] = float(np.linalg.norm(G))
        st["newton_iters"] += 1
        if st["norm_dx"] < tol and st["norm_G"] < tol:
            st["converged"] = 1
            break
        if st["norm_dx"] > 1e2:
            break
    return xc, st
