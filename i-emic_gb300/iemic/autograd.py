"""torch.autograd bridge for gradient checks of the steady-state adjoint.

``SteadyPsiMax.apply(field, ocean, name, x0)`` sets the surface forcing field
``name`` (an (m, n) tensor) on the ocean, converges the steady state with
Newton from ``x0`` and returns g = max psi_M (Sv); its backward pass is the
adjoint gradient of iemic_adjoint_psim (one transposed solve with the
preconditioner of J). The wrapper exists for gradient checks only (finite
differences, torch.autograd.gradcheck-style comparisons); the computation is
the library's.
"""
import numpy as np
import torch


class SteadyPsiMax(torch.autograd.Function):
    @staticmethod
    def forward(ctx, field, ocean, name, x0, newton_tol=1e-10, precision=1):
        f = field.detach().cpu().numpy().astype(np.float64)
        ocean.setForcing(**{name: f.ravel()})
        x, st = ocean.newton(np.asarray(x0), precision=precision, max_iters=20, tol=newton_tol)
        if st["status"] != 0:
            raise RuntimeError("Newton did not converge: %s" % st)
        g, grads, _, _ = ocean.adjointPsiM(x, precision=precision)
        ctx.grad = torch.as_tensor(grads[name], dtype=field.dtype)
        return torch.as_tensor(g, dtype=field.dtype)

    @staticmethod
    def backward(ctx, grad_out):
        return grad_out * ctx.grad, None, None, None, None, None
