#!/usr/bin/env python3
"""Generate haadf_cfg0_converged.npz: the reference-order reconstruction of the benchmark's small
HAADF configuration run to convergence, the fixture of the converged-volume check.

Made by the oracle (oracle/mbir_oracle.c), which reproduces the reference's own programs bit for
bit (tests/test_oracle_vs_ref.py, including this configuration's output digests after 1, 5 and
20 outer iterations).  The reference's command-line programs cannot run this case themselves:
it needs ZERO_SKIPPING = 0, an AdvancedParameters field that the engines set to 1
(HAADF_ReconstructionEngine.cpp:255) and no flag exposes.  Zero skipping is off because with it
the ICD fixed point depends on the visit order (a voxel at zero whose neighbours are all zero is
never revisited), so two reference runs that seed their visit orders differently do not converge
to the same volume; without it every order converges to the MAP estimate.

The run: volume 128 x 32 x 64, 71 views over +-70 deg, thickness 32, sigma_x 0.2, diffuseness
0.1, gain/offset and variance estimation on, one ICD sweep per outer iteration in the
reference's visit order with a new seed per sweep (seed + k, as the reference's clock seed
changes between sweeps), 500 outer iterations.  Stored: the volume (float32, z x y), gains,
offsets, variances and the MAP cost.

Usage: python tests/golden/make_converged.py   (about four minutes on one core)
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (os.path.join(ROOT, "oracle"), os.path.join(ROOT, "openmbir-tem_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)

import oracle  # noqa: E402
import refrun  # noqa: E402
import synthetic  # noqa: E402

SEED = 12345
OUTER = 500


def main():
    y, ang, _ = synthetic.haadf_two_spheres()
    o = refrun.haadf_params(32.0, 0.1, 0.2, OUTER)
    o.zero_skipping = 0
    orc = oracle.Oracle(o, y, ang, refrun.REF_DELTA, refrun.REF_DELTA)
    orc.prepare()
    n, _ = orc.run(SEED, 0, 1)
    assert n == OUTER, n
    cost = orc.cost()[0]
    path = os.path.join(HERE, "haadf_cfg0_converged.npz")
    np.savez_compressed(path, volume_zxy=orc.volume().astype(np.float32), gain=orc.gain(),
                        offset=orc.offset(), variance=orc.variance(), cost=np.float64(cost),
                        outer=np.int32(OUTER), seed=np.int32(SEED))
    print("haadf_cfg0_converged.npz", os.path.getsize(path), "cost", cost)
    return 0


if __name__ == "__main__":
    sys.exit(main())
