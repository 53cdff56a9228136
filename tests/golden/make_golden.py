"""Regenerate the golden fixtures of tests/golden/ (run from the repository root).

1. mask_global_96x38x12.npy: the reference's real-continent land mask
   data/mkmask/mask_global_96x38x12 (read only when ``--reference PATH`` names
   a checkout of the reference), converted with the reader rules of readmask
   (src/ocean/topo.F90:41-60): per level k = 0..l+1 a header line, then rows
   j = m+1 down to 0 of n+2 digits (i = 0..n+1). Stored as int8 in the
   (l+2, m+2, n+2) layout of the C ABI (i fastest). mask_natl8.npy: the 8x8x4
   North-Atlantic mask of the reference's src/tests/test_ocean.C, the same way.
2. oracle_box_seed0.npz / oracle_glob24_seed1.npz: values of the CPU oracle
   at seeded states -- F, J 1, J^T 1, every 97th value of J in the maximal
   graph and a SHA-256 of the graph's index arrays -- so that the oracle and
   the GPU path are both pinned to fixed numbers across machines.
"""
import hashlib
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
HERE = os.path.dirname(os.path.abspath(__file__))
sys.path[:0] = [ROOT, os.path.join(ROOT, "i-emic_gb300"), os.path.join(ROOT, "tests")]


def read_mask(path, n, m, l):
    lines = open(path).read().splitlines()
    lm = np.ones((l + 2, m + 2, n + 2), dtype=np.int8)
    q = 0
    for k in range(l + 2):
        q += 1   # header line
        for j in range(m + 1, -1, -1):
            row = lines[q]
            q += 1
            lm[k, j, :] = [int(ch) for ch in row[:n + 2]]
    return lm


def oracle_summary(o, x):
    import scipy.sparse as sp
    rp, ci = o.graph()
    vals, _ = o.jacobian(x)
    J = sp.csr_matrix((vals, ci, rp), shape=(o.ndim, o.ndim))
    one = np.ones(o.ndim)
    h = hashlib.sha256(rp.astype(np.int32).tobytes() + ci.astype(np.int32).tobytes()).hexdigest()
    return dict(F=o.rhs(x), J1=J @ one, JT1=J.T @ one, Jsample=vals[::97].copy(), graph_sha256=np.array(h))


def main():
    import argparse
    from helpers import box_case, global_case, make_oracle, seeded_state
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=None, help="root of the reference checkout (for the real-continent mask)")
    args = ap.parse_args()
    ref_mask = None if args.reference is None else os.path.join(args.reference, "data", "mkmask",
                                                                 "mask_global_96x38x12")
    if ref_mask is not None and os.path.exists(ref_mask):
        np.save(os.path.join(HERE, "mask_global_96x38x12.npy"), read_mask(ref_mask, 96, 38, 12))
        # the mask of src/tests/test_ocean.C (test/ocean/ocean_params.xml: 8x8x4 North Atlantic)
        np.save(os.path.join(HERE, "mask_natl8.npy"),
                read_mask(os.path.join(args.reference, "data", "mkmask", "mask_natl8"), 8, 8, 4))
    for name, case, seed in (("box_seed0", box_case, 0), ("glob24_seed1", global_case, 1)):
        cfg, lm, frc = case()
        o = make_oracle(cfg, lm, frc)
        x = seeded_state(cfg, seed, uvw=0.01)
        np.savez_compressed(os.path.join(HERE, "oracle_%s.npz" % name), **oracle_summary(o, x))


if __name__ == "__main__":
    main()
