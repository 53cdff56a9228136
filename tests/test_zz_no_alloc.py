"""iemic_rhs_dev_noalloc against iemic_rhs_dev (collected last on purpose:
it must pass alone and after every other test in the process).

Two calls in a row on the same handle, each compared bit for bit with the
handle-scratch entry point, on the 16x16x4 box, a 24x12x6 periodic global
ocean and the 16x16x16 gateway basin with vertical mixing (whose partition
control also keeps its partial sums in the static array) and the 8x8x4
North-Atlantic basin with the integral condition on S and fixed pressure
points; calls on two
handles back to back, read on another stream right after each returns; a
grid whose padded fields exceed the static scratch is rejected without
touching the output.
"""
import ctypes

import numpy as np
import pytest

from helpers import box_case, gateway_case, global_case, make_gpu, natl8_case, seeded_state

pytestmark = pytest.mark.gpu


def _dev(a):
    import torch
    return torch.tensor(a, dtype=torch.float64, device="cuda")


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def _gateway():
    return gateway_case(2)


def _natl8():
    return natl8_case(0, 1)


@pytest.mark.parametrize("case", [box_case, global_case, _gateway, _natl8])
def test_noalloc_rhs_matches_rhs_dev_twice(case):
    import torch
    from iemic import workloads as W
    cfg, lm, frc = case()
    g = make_gpu(cfg, lm, frc, W.GATEWAY_STARTING_PARAMETERS if cfg.get("vmix") else W.STARTING_PARAMETERS)
    g.setPar("Combined Forcing", 0.5)
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


def test_noalloc_two_handles_back_to_back():
    """Each call has finished when it returns: the result is read at once on
    torch's stream (not the handle's), and the next call, on another handle,
    reuses the shared array."""
    import torch
    cases = [box_case(), global_case()]
    hs = [make_gpu(*c) for c in cases]
    xs = [_dev(seeded_state(c[0], 4 + q, uvw=0.01)) for q, c in enumerate(cases)]
    refs = []
    for g, x in zip(hs, xs):
        F = torch.zeros(g.ndim, dtype=torch.float64, device="cuda")
        assert g.L.iemic_rhs_dev(g.handle, _ptr(x), _ptr(F)) == 0
        refs.append(F.cpu().numpy())
    for _ in range(2):
        got = []
        for g, x in zip(hs, xs):
            F = torch.full((g.ndim,), np.nan, dtype=torch.float64, device="cuda")
            torch.cuda.synchronize()
            assert g.L.iemic_rhs_dev_noalloc(g.handle, _ptr(x), _ptr(F)) == 0
            got.append(F.clone())          # ordered on torch's stream, after the call returned
        for r, F in zip(refs, got):
            assert np.array_equal(r.view(np.int64), F.cpu().numpy().view(np.int64))


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
