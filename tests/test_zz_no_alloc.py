"""iemic_rhs_dev_noalloc against iemic_rhs_dev (collected last on purpose:
it must pass alone and after every other test in the process).

Two calls in a row on the same handle, each compared bit for bit with the
handle-scratch entry point, on the 16x16x4 box and a 24x12x6 periodic
global ocean; a grid whose padded fields exceed the static scratch is
rejected without touching the output.
"""
import ctypes

import numpy as np
import pytest

from helpers import box_case, global_case, make_gpu, seeded_state

pytestmark = pytest.mark.gpu


def _dev(a):
    import torch
    return torch.tensor(a, dtype=torch.float64, device="cuda")


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


@pytest.mark.parametrize("case", [box_case, global_case])
def test_noalloc_rhs_matches_rhs_dev_twice(case):
    import torch
    cfg, lm, frc = case()
    g = make_gpu(cfg, lm, frc)
    L = g.L
    for seed in (0, 1):   # two calls in a row, different states
        x = _dev(seeded_state(cfg, seed, uvw=0.01))
        F_ref = torch.zeros(g.ndim, dtype=torch.float64, device="cuda")
        F_na = torch.full((g.ndim,), np.nan, dtype=torch.float64, device="cuda")
        assert L.iemic_rhs_dev(g.handle, _ptr(x), _ptr(F_ref)) == 0
        assert L.iemic_rhs_dev_noalloc(g.handle, _ptr(x), _ptr(F_na)) == 0
        torch.cuda.synchronize()
        a, b = F_ref.cpu().numpy(), F_na.cpu().numpy()
        assert np.array_equal(a.view(np.int64), b.view(np.int64))
        assert np.linalg.norm(a) > 0


def test_noalloc_rejects_grids_over_the_scratch():
    import torch
    cfg, lm, frc = global_case(n=100, m=100, l=10)   # 102*102*12 padded cells > 65536
    g = make_gpu(cfg, lm, frc)
    x = torch.zeros(g.ndim, dtype=torch.float64, device="cuda")
    F = torch.full((g.ndim,), 7.0, dtype=torch.float64, device="cuda")
    assert g.L.iemic_rhs_dev_noalloc(g.handle, _ptr(x), _ptr(F)) == -1
    torch.cuda.synchronize()
    assert bool((F == 7.0).all())
    assert g.L.iemic_rhs_dev_noalloc(None, _ptr(x), _ptr(F)) == -1
