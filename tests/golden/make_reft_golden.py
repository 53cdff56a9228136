"""Regenerate tests/golden/reft_ocean_reference.npz (run from the repository root).

Reads, from a checkout of the reference (``--reference PATH``):
- test/ocean/ocean_reference.h5: the state the reference's own test
  src/tests/reft_ocean.C compares against (a continuation in Combined Forcing
  0 -> 0.02 on the 16x16x16 gateway basin with vertical mixing, Mixing = 2,
  test/ocean/reft_ocean_params.xml and reft_continuation_params.xml), read with
  the pure-Python HDF5 reader h5lite.py. Kept: State/Values (24,576 FP64
  values), the final Combined Forcing, the land mask THCM used
  (MaskGlobal/Global) and the parameter vector stored with the state;
- data/mkmask/mask_gateway, converted by the readmask rules
  (src/ocean/topo.F90:41-60) exactly as make_golden.read_mask does, and
  checked against MaskGlobal/Global.
"""
import argparse
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", required=True, help="root of the reference checkout")
    args = ap.parse_args()
    import h5lite
    from make_golden import read_mask
    d = h5lite.read(os.path.join(args.reference, "test", "ocean", "ocean_reference.h5"))
    mask = read_mask(os.path.join(args.reference, "data", "mkmask", "mask_gateway"), 16, 16, 16)
    landm = d["MaskGlobal/Global"].astype(np.int8).reshape(18, 18, 18)
    if not np.array_equal(mask, landm):
        raise SystemExit("mask_gateway conversion differs from the reference's MaskGlobal/Global")
    params = {k.split("/", 1)[1]: float(v) for k, v in d.items() if k.startswith("Parameters/")}
    np.savez_compressed(os.path.join(HERE, "reft_ocean_reference.npz"),
                        state=d["State/Values"].ravel().astype(np.float64), landm=landm,
                        par_names=np.array(sorted(params)), par_values=np.array([params[k] for k in sorted(params)]))


if __name__ == "__main__":
    main()
