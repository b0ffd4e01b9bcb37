"""Convert the reference's CDKLM16 regression vectors into a compact fixture.

Reads ``test/timestep50/CDKLM16_*_{eta,u,v}.dat`` from a checkout of the
reference (the first argument, or ``$GPUOCEAN_REFERENCE``) and writes the interior (70 x 50) of
each field as float32 into ``cdklm16_timestep50.npz`` next to this script.
The ``.dat`` files hold float32 GPU results printed as float64 text, so the
float32 round trip is exact.  The ``u``/``v`` files hold hu/hv.

Usage:  python tests/golden/make_timestep50.py REFERENCE_ROOT
"""
import os
import sys

import numpy as np

CASES = ["wallBC_central", "wallBC_corner", "wallBC_upperCorner",
         "periodic_corner", "periodic_upperCorner",
         "periodicNS_corner", "periodicNS_upperCorner",
         "periodicEW_corner", "periodicEW_upperCorner",
         "coriolis_central", "betamodel_central", "wallBC_central_bathymetry"]


def main():
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("GPUOCEAN_REFERENCE")
    if not root:
        sys.exit("usage: %s REFERENCE_ROOT (or set GPUOCEAN_REFERENCE)" % sys.argv[0])
    src = os.path.join(root, "test", "timestep50")
    out = {}
    for case in CASES:
        for field in ("eta", "u", "v"):
            if case.endswith("_bathymetry"):
                name = "CDKLM16_" + case[:-len("_bathymetry")] + "_bathymetry_" + field + ".dat"
            else:
                name = "CDKLM16_" + case + "_" + field + ".dat"
            a = np.loadtxt(os.path.join(src, name))
            assert a.shape == (74, 54), (name, a.shape)
            a32 = a.astype(np.float32)
            assert np.array_equal(a32.astype(np.float64), a), name
            out[case + "/" + field] = a32[2:-2, 2:-2]
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "cdklm16_timestep50.npz")
    np.savez_compressed(dst, **out)
    print("wrote", dst, sum(v.nbytes for v in out.values()), "bytes raw")


if __name__ == "__main__":
    main()
