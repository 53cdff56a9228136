"""Shared builders for the test suite: the same seeded workloads on the
oracle (CPU, checker only) and on the GPU engine."""
import os

import numpy as np

from iemic import workloads as W

ORACLE_PAR = {"Combined Forcing": "COMB", "Temperature Forcing": "TEMP",
              "Salinity Forcing": "SALT", "Wind Forcing": "WIND", "Solar Forcing": "SUNP",
              "SPL1": "SPL1", "SPL2": "SPL2"}
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def gateway_case(vmix=2):
    """The reference's regression case (reft_ocean) with the land mask THCM
    used, as stored in test/ocean/ocean_reference.h5."""
    g = np.load(os.path.join(GOLDEN, "reft_ocean_reference.npz"))
    cfg = dict(W.gateway_16x16x16(), vmix=vmix)
    return cfg, g["landm"].astype(np.int32), None


def natl8_case(sres=0, fix_pressure_points=0):
    """The reference's src/tests/test_ocean.C ocean (mask_natl8, SRES = 0)."""
    lm = np.load(os.path.join(GOLDEN, "mask_natl8.npy")).astype(np.int32)
    return dict(W.natl8_8x8x4(), sres=sres, fix_pressure_points=fix_pressure_points), lm, None


def gateway_golden():
    g = np.load(os.path.join(GOLDEN, "reft_ocean_reference.npz"))
    pars = dict(zip([str(s) for s in g["par_names"]], g["par_values"]))
    return g["state"], pars


def box_case():
    cfg = W.box_16x16x4()
    return cfg, None, W.box_forcing(cfg)


def global_case(n=24, m=12, l=6, seed=3):
    """A small periodic global ocean with seeded land and stretched levels."""
    cfg = dict(W.global_96x38x12(), n=n, m=m, l=l)
    return cfg, W.seeded_global_mask(cfg, seed), None


def make_oracle(cfg, landm, forcing, params=W.STARTING_PARAMETERS):
    import oracle
    o = oracle.Oracle(cfg, landm)
    if forcing:
        o.set_forcing(**forcing)
    for name, v in params:
        o.set_par(ORACLE_PAR[name], v)
    return o


def make_gpu(cfg, landm, forcing, params=W.STARTING_PARAMETERS):
    from iemic import Ocean
    return Ocean(cfg, landm, forcing=forcing, starting_parameters=params)


def seeded_state(cfg, seed, uvw=0.0):
    x = W.rest_state_with_ts_noise(cfg, seed)
    if uvw:
        rng = np.random.default_rng(seed + 1000)
        nc = x.size // 6
        for t in (0, 1, 2, 3):
            x[t::6] = rng.normal(0.0, uvw, nc)
    return x
