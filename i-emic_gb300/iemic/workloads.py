"""Seeded synthetic THCM ocean workloads.

Each workload mirrors the THCM XML keys the reference reads
(src/ocean/THCM.C:180-260) plus a land mask in the reference's ``readmask``
layout (src/ocean/topo.F90:41-60: (n+2)(m+2)(l+2) integers, i fastest,
0 = ocean, 1 = land, 3 = periodic border) and the injected forcing fields of
``m_inserts`` (src/ocean/inserts.F90). The reference's Levitus/Trenberth data
files are not available, so the idealized profiles or seeded fields stand in.
"""
import numpy as np

OCEAN, LAND, PERIO = 0, 1, 3

BASE = dict(xmin_deg=286.0, xmax_deg=350.0, ymin_deg=10.0, ymax_deg=74.0, periodic=0,
            hdim=4000.0, qz=1.0, alphaT=1.0e-4, alphaS=7.6e-4, ih=0, coriolis_on=1,
            tres=1, sres=1, iza=2, ite=1, its=1, forcing_type=0, vmix=0, rho_mixing=0, tap=1,
            sint_sign=-1, intcon_i=-1, intcon_j=-1, fix_pressure_points=0)


def gateway_16x16x16():
    """The reference's regression case (test/ocean/reft_ocean_params.xml,
    driven by src/tests/reft_ocean.C): 16x16x16 cells, lon 300-340, lat 20-60,
    periodic, depth 4000 m, uniform levels, the land mask data/mkmask/mask_gateway
    (a basin with a periodic channel along its southern edge), vertical
    mixing with adaptive partitioning (Mixing = 2, Taper 1, no Rho Mixing),
    Forcing Type 2, idealized wind and T/S restoring."""
    return dict(BASE, n=16, m=16, l=16, xmin_deg=300.0, xmax_deg=340.0, ymin_deg=20.0, ymax_deg=60.0,
                periodic=1, hdim=4000.0, qz=1.0, iza=2, ite=1, its=1, forcing_type=2, vmix=2, rho_mixing=0,
                tap=1)


def natl8_8x8x4():
    """The reference's unit-test ocean (test/ocean/ocean_params.xml, driven by
    src/tests/test_ocean.C): 8x8x4 cells, lon 286-350, lat 10-74, depth 4000 m,
    the land mask data/mkmask/mask_natl8, fixed-partition vertical mixing
    (Mixing = 1), T restoring, no S restoring (SRES = 0: the integral
    condition on S), idealized forcing."""
    return dict(BASE, n=8, m=8, l=4, periodic=0, vmix=1, rho_mixing=0, tap=1, tres=1, sres=0, iza=2, ite=1, its=1,
                forcing_type=0)


NATL8_STARTING_PARAMETERS = (("Combined Forcing", 0.0), ("Solar Forcing", 0.0), ("Salinity Forcing", 1.0),
                             ("Wind Forcing", 1.0), ("Temperature Forcing", 10.0), ("SPL1", 2.0e3),
                             ("SPL2", 0.01))


# "Starting Parameters" of test/ocean/reft_ocean_params.xml
GATEWAY_STARTING_PARAMETERS = (("Combined Forcing", 0.0), ("Solar Forcing", 0.0), ("Salinity Forcing", 0.1),
                               ("Wind Forcing", 1.0), ("Temperature Forcing", 10.0), ("SPL1", 2.0e3),
                               ("SPL2", 0.01))
# test/ocean/reft_continuation_params.xml (with getDefaultInitParameters for
# the keys it leaves out)
GATEWAY_CONTINUATION = dict(ds=2.0e-3, ds_min=1.0e-8, ds_max=1.0e-1, destination=0.02, max_steps=20,
                            opt_newton=3.0, newton_tol=1.0e-2, destination_tol=1.0e-4, epsilon=1.0e-5,
                            tan_scaling=1.0e-3, newton_chord=0, predictor_bound=3000.0)


def box_16x16x4():
    """16x16x4 idealized North-Atlantic box (lon 286-350, lat 10-74), flat
    bottom at 4000 m, no land, injected forcing: taux = cos(pi*lat/60) (the
    0.1 N/m^2 scale is carried by par(AL_T), src/ocean/usrc.F90:1164), tauy = 0,
    restoring T* and S* linear in latitude (+1 at 10N to -1 at 74N)."""
    cfg = dict(BASE, n=16, m=16, l=4, iza=3, ite=2, its=2)
    return cfg


def _grid_lat(cfg):
    m = cfg["m"]
    ymin, ymax = np.radians(cfg["ymin_deg"]), np.radians(cfg["ymax_deg"])
    dy = (ymax - ymin) / m
    y = (np.arange(1, m + 1) - 0.5) * dy + ymin
    yv = np.arange(1, m + 1) * dy + ymin
    return np.degrees(y), np.degrees(yv)


def box_forcing(cfg):
    n, m = cfg["n"], cfg["m"]
    lat, latv = _grid_lat(cfg)
    taux = np.repeat(np.cos(np.pi * latv / 60.0)[:, None], n, axis=1).ravel()
    ramp = 1.0 - 2.0 * (lat - cfg["ymin_deg"]) / (cfg["ymax_deg"] - cfg["ymin_deg"])
    tatm = np.repeat(ramp[:, None], n, axis=1).ravel()
    return dict(taux=taux, tauy=np.zeros(n * m), tatm=tatm, emip=tatm.copy())


STARTING_PARAMETERS = (("Combined Forcing", 1.0), ("Temperature Forcing", 10.0),
                       ("Salinity Forcing", 0.1), ("Wind Forcing", 1.0))


def rest_state_with_ts_noise(cfg, seed, sigma=0.1):
    """u,v,w,p = 0; T,S ~ N(0, sigma^2) from numpy.random.default_rng(seed)."""
    nc = cfg["n"] * cfg["m"] * cfg["l"]
    rng = np.random.default_rng(seed)
    x = np.zeros(6 * nc)
    x[4::6] = rng.normal(0.0, sigma, nc)
    x[5::6] = rng.normal(0.0, sigma, nc)
    return x


def _smooth_periodic(field, passes, periodic_x):
    f = field.copy()
    for _ in range(passes):
        if periodic_x:
            f = (f + np.roll(f, 1, axis=1) + np.roll(f, -1, axis=1)) / 3.0
        else:
            g = f.copy()
            g[:, 1:-1] = (f[:, :-2] + f[:, 1:-1] + f[:, 2:]) / 3.0
            f = g
        g = f.copy()
        g[1:-1, :] = (f[:-2, :] + f[1:-1, :] + f[2:, :]) / 3.0
        f = g
    return f


def _largest_component(ocean2d, periodic_x):
    """Keep only the ocean component with the most cells (4-connectivity),
    like the reference's flood fill in src/ocean/topo.F90 (depth3land)."""
    m, n = ocean2d.shape
    label = -np.ones((m, n), dtype=np.int64)
    best, best_size, cur = -1, 0, 0
    for j0 in range(m):
        for i0 in range(n):
            if not ocean2d[j0, i0] or label[j0, i0] >= 0:
                continue
            stack = [(j0, i0)]
            label[j0, i0] = cur
            size = 0
            while stack:
                j, i = stack.pop()
                size += 1
                for dj, di in ((1, 0), (-1, 0), (0, 1), (0, -1)):
                    jj, ii = j + dj, i + di
                    if periodic_x:
                        ii %= n
                    if 0 <= jj < m and 0 <= ii < n and ocean2d[jj, ii] and label[jj, ii] < 0:
                        label[jj, ii] = cur
                        stack.append((jj, ii))
            if size > best_size:
                best, best_size = cur, size
            cur += 1
    return label == best


def seeded_global_mask(cfg, seed, land_fraction=0.30, min_depth_frac=0.3):
    """Seeded land mask: smoothed N(0,1) blobs thresholded for about
    ``land_fraction`` surface land, a smooth random bathymetry between
    ``min_depth_frac``*hdim and hdim, levels from the stretched grid
    (a cell is ocean where its centre z(k) lies above the bottom, the rule of
    src/ocean/topo.F90 depth3land), one connected basin, periodic borders
    marked 3 where the wrapped neighbour is water."""
    n, m, l = cfg["n"], cfg["m"], cfg["l"]
    periodic = bool(cfg["periodic"])
    rng = np.random.default_rng(seed)
    blobs = _smooth_periodic(rng.normal(size=(m, n)), 6, periodic)
    thr = np.quantile(blobs, 1.0 - land_fraction)
    ocean = blobs < thr
    ocean = _largest_component(ocean, periodic)
    bath = _smooth_periodic(rng.normal(size=(m, n)), 4, periodic)
    bath = (bath - bath.min()) / max(bath.max() - bath.min(), 1e-30)
    depth = cfg["hdim"] * (min_depth_frac + (1.0 - min_depth_frac) * bath)   # metres
    # cell-centre depths z(k) (src/ocean/grid.F90 fz)
    qz = cfg["qz"]
    dz = 1.0 / l
    ze = (np.arange(1, l + 1) - 0.5) * dz - 1.0
    if qz > 1.0:
        zc = -1.0 + np.tanh(qz * (ze + 1.0)) / np.tanh(qz)
    else:
        zc = ze + (1.0 - qz) * ze * (1.0 - ze)
    lm = np.full((l + 2, m + 2, n + 2), LAND, dtype=np.int32)
    for k in range(1, l + 1):
        wet = ocean & (zc[k - 1] * cfg["hdim"] > -depth)
        lm[k, 1:m + 1, 1:n + 1] = np.where(wet, OCEAN, LAND)
    # one connected basin at every level is not required, but the surface must be
    # connected; deeper isolated pockets stay (they are connected vertically).
    if periodic:
        lm[:, :, 0] = np.where(lm[:, :, n] == LAND, LAND, PERIO)
        lm[:, :, n + 1] = np.where(lm[:, :, 1] == LAND, LAND, PERIO)
        lm[0, :, :] = LAND
        lm[l + 1, :, :] = LAND
        lm[:, 0, :] = LAND
        lm[:, m + 1, :] = LAND
    return lm.ravel()


def global_96x38x12():
    """Global 4-degree ocean: 96x38x12, lon 0-360 periodic, lat +-81,
    depth 5000 m, stretched levels qz = 2.25 (run/ocean/global/ocean_params.xml),
    idealized forcing (Bryan wind profile, cos(pi y/ymax) restoring)."""
    return dict(BASE, n=96, m=38, l=12, xmin_deg=0.0, xmax_deg=360.0, ymin_deg=-81.0,
                ymax_deg=81.0, periodic=1, hdim=5000.0, qz=2.25, iza=2, ite=1, its=1)


def global_360x160x20():
    """1-degree ocean: 360x160x20, lat +-80, depth 5000 m (stretched)."""
    return dict(BASE, n=360, m=160, l=20, xmin_deg=0.0, xmax_deg=360.0, ymin_deg=-80.0,
                ymax_deg=80.0, periodic=1, hdim=5000.0, qz=2.25, iza=2, ite=1, its=1)


def global_180x76x16():
    """2-degree ocean: 180x76x16, lat +-76, depth 5000 m (stretched)."""
    return dict(BASE, n=180, m=76, l=16, xmin_deg=0.0, xmax_deg=360.0, ymin_deg=-76.0,
                ymax_deg=76.0, periodic=1, hdim=5000.0, qz=2.25, iza=2, ite=1, its=1)


def global_360x160x20():
    """Global 1-degree ocean: 360x160x20, lon 0-360 periodic, lat +-80,
    depth 5000 m, stretched levels qz = 2.25; used with a seeded mask whose
    smooth bathymetry spans 500-5000 m (``seeded_global_mask(cfg, seed,
    min_depth_frac=0.1)``)."""
    return dict(BASE, n=360, m=160, l=20, xmin_deg=0.0, xmax_deg=360.0, ymin_deg=-80.0,
                ymax_deg=80.0, periodic=1, hdim=5000.0, qz=2.25, iza=2, ite=1, its=1)
