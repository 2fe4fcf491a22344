#!/usr/bin/env python3
"""Generate the reference-output fixtures in this directory from OpenMBIR-TEM itself.

Needs the reference tree (its programs are built from source by oracle/build_ref.py into
oracle/_ref) and runs them through oracle/refrun.py on seeded synthetic inputs:

* haadf_small.npz -- a reduced HAADF case (64 x 8 detector, 36 views over +-70 deg, thickness
  16): the forward projection of a random volume (0 outer iterations from
  --initial_recon_file; the volume's values are float32 numbers) and 5 outer iterations with
  gain/offset and variance estimation;
* bf_small.npz -- a reduced bright-field case (64 x 8 detector, 31 views over +-60 deg): 40
  outer iterations with 3 inner calls (the Bragg schedule: T = 5e10 for the first calls, then
  T = 3), NHICD lists, offset and variance estimation; and the first 6 calls of the same
  schedule (4 outer iterations);
* output_headers.json -- the headers of the reference's MRC, VTK and Avizo volume files for the
  reduced HAADF case (everything but the voxel values);
* haadf_bf_assist_small.npz -- the reduced HAADF case with a bright-field tilt series of the
  same size (--brightfield; the bright-field counts seen through one of the case's spheres):
  5 outer iterations;
* bf_multires_small.npz -- the reduced bright-field case with 12 detector rows over two
  resolution levels (coarse 2x, then 1x), 2 outer iterations with 2 inner calls at the coarse
  level;
* shepp_logan.npz -- the reference's own input fixture (Resources/InputFiles/
  ScheppLoganSinogram128NoiselessLimitedAngle.bin, 87 views over +-70 deg at 1 deg steps near
  the ends and 2 deg in the middle, as ParamsWithROIAndViewSelectShepLogan.txt lists them; 128
  x 3 detector) reconstructed with thickness 32 from the fixture's offsets (0, the default
  offset; the offset the reference estimates from this noiseless sinogram's view means leaves
  an all-zero first sweep and NaN gains), 3 outer iterations with gain/offset and variance
  estimation;
* haadf_cfg0.json -- the benchmark's small HAADF configuration (128 x 32 detector, 71 views over
  +-70 deg at 2 deg, thickness 32, volume 128 x 32 x 64): SHA-256 digests and sums of the
  inputs and of the reference's float64 outputs after 1, 5 and 20 outer iterations.

Every run uses one worker and a frozen clock seed (refrun.py explains both).  The inputs of the
small cases are stored with their outputs; the cfg0 input is regenerated from its seed and
checked against its stored digest.

Usage: python tests/golden/make_golden.py [fixture ...]   (default: all; names without suffix)
"""
import hashlib
import json
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (os.path.join(ROOT, "oracle"), os.path.join(ROOT, "openmbir-tem_gb300"),
          os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)

import refrun  # noqa: E402
import synthetic  # noqa: E402
from conftest import bf_case, small_case  # noqa: E402

HAADF_SEED = 12345
BF_SEED = 777


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a, "<f8").tobytes()).hexdigest()


def cfg0_input():
    y, ang, _ = synthetic.haadf_two_spheres()
    return y, ang


def output_headers(tmp):
    """The headers of the reference's volume files (MRC with its FEI extended header, VTK, Avizo)
    for the reduced HAADF case, 1 outer iteration: everything but the voxel values."""
    y, ang, th = small_case()
    refrun.run_haadf(os.path.join(tmp, "hdr"), y, ang, th, 0.1, 0.2, 1, seed=HAADF_SEED)
    out = os.path.join(tmp, "hdr", "out")
    with open(os.path.join(out, "recon.mrc"), "rb") as f:
        mrc = f.read(1024)
        n_ext = int.from_bytes(mrc[92:96], "little")
        ext = f.read(n_ext)
    with open(os.path.join(out, "recon.vtk"), "rb") as f:
        vtk = f.read()
    vtk_hdr = vtk[:vtk.index(b"LOOKUP_TABLE default\n") + len(b"LOOKUP_TABLE default\n")]
    with open(os.path.join(out, "recon.am"), "rb") as f:
        am = f.read()
    am_hdr = am[:am.index(b"# Data section follows\n@1\n") + len(b"# Data section follows\n@1\n")]
    rec = {"mrc_header_hex": mrc.hex(), "mrc_ext_header_hex": ext.hex(),
           "mrc_size": os.path.getsize(os.path.join(out, "recon.mrc")),
           "vtk_header": vtk_hdr.decode(), "vtk_size": len(vtk),
           "am_header": am_hdr.decode(), "am_size": len(am)}
    with open(os.path.join(HERE, "output_headers.json"), "w") as f:
        json.dump(rec, f, indent=1, sort_keys=True)


def haadf_small(tmp):
    y, ang, th = small_case()
    n_theta, n_r, n_t = y.shape
    kw = dict(thickness=th, diffuseness=0.1, sigma_x=0.2, seed=HAADF_SEED)
    rng = np.random.default_rng(11)
    n_z = int(round(2 * th))
    init_yxz = np.maximum(rng.normal(0.3, 0.3, (n_t, n_r, n_z)), 0.0).astype(np.float32)
    fp = refrun.run_haadf(os.path.join(tmp, "hs_fp"), y, ang, outer=0,
                          initial=init_yxz.astype(np.float64), **kw)
    it5 = refrun.run_haadf(os.path.join(tmp, "hs_it5"), y, ang, outer=5, **kw)
    np.savez_compressed(os.path.join(HERE, "haadf_small.npz"), counts=y, tilts=ang,
                        thickness=th, init_yxz=init_yxz, fp_sinogram=fp["sinogram"],
                        it5_object_yxz=it5["object_yxz"], it5_gain=it5["gain"],
                        it5_offset=it5["offset"])


def shepp_logan_input(reference=refrun.DEFAULT_REFERENCE):
    """The reference's Shepp-Logan sinogram (float64 [theta][r][t], 87 x 128 x 3) as float32
    counts, and its tilt angles (the parameter file lists each angle followed by its selection
    flag, all 1)."""
    d = os.path.join(reference, "Resources", "InputFiles")
    sino = np.fromfile(os.path.join(d, "ScheppLoganSinogram128NoiselessLimitedAngle.bin"), "<f8")
    with open(os.path.join(d, "ParamsWithROIAndViewSelectShepLogan.txt")) as f:
        text = f.read()
    body = text.split("SinoAngles", 1)[1].split("Geom", 1)[0].split()
    angles = np.array([float(a) for a in body[0::2]], np.float32)
    assert angles.size == 87 and all(v == "1" for v in body[1::2])
    return sino.reshape(87, 128, 3).astype(np.float32), angles


def shepp_logan(tmp):
    y, ang = shepp_logan_input()
    th = 32.0
    out = refrun.run_haadf(os.path.join(tmp, "sl"), y, ang, th, 0.1, 0.2, 3, seed=HAADF_SEED,
                           extra=("--use_default_offset", "--default_offset", "0"))
    np.savez_compressed(os.path.join(HERE, "shepp_logan.npz"), counts=y, tilts=ang,
                        thickness=th, it3_object_yxz=out["object_yxz"], it3_gain=out["gain"],
                        it3_offset=out["offset"])


def haadf_bf_assist_small(tmp):
    """The reduced HAADF case with a bright-field tilt series of the same size (--brightfield):
    5 outer iterations."""
    y, ang, th = small_case()
    bf = bright_field_series(y.shape, ang)
    out = refrun.run_haadf(os.path.join(tmp, "hbf"), y, ang, th, 0.1, 0.2, 5, seed=HAADF_SEED,
                           brightfield=bf)
    np.savez_compressed(os.path.join(HERE, "haadf_bf_assist_small.npz"), counts=y, bf_counts=bf,
                        tilts=ang, thickness=th, it5_object_yxz=out["object_yxz"],
                        it5_gain=out["gain"], it5_offset=out["offset"])


def bf_multires_small(tmp):
    """The reduced bright-field case (12 detector rows) over two resolution levels (coarse 2x,
    then 1x), 2 outer iterations with 2 inner calls at the coarse level.  (The reference's HAADF
    program stops at its second level: it reads a FinalVariances.bin that its first level does
    not write.)"""
    c, ang, th = bf_case(n_t=12)
    out = refrun.run_bf(os.path.join(tmp, "bmr"), c, ang, th, 0.1, 0.02, outer=2, inner=2,
                        seed=BF_SEED, levels=2)
    np.savez_compressed(os.path.join(HERE, "bf_multires_small.npz"), counts=c, tilts=ang,
                        thickness=th, object_yxz=out["object_yxz"], offset=out["offset"],
                        variance=out["variance"])


def bright_field_series(shape, ang, seed=5):
    """Bright-field counts seen through the first sphere of the reduced HAADF case."""
    rng = np.random.default_rng(seed)
    proj = synthetic.ellipsoid_projection(ang, shape[1], shape[2],
                                          [(-12.0, 0.0, 0.0, 10.0, 10.0, 10.0, 1.0)])
    return np.maximum(rng.poisson(1.0e4 * np.exp(-0.02 * proj)), 1).astype(np.float32)


def bf_small(tmp):
    c, ang, th = bf_case()
    out = refrun.run_bf(os.path.join(tmp, "bf40"), c, ang, th, 0.1, 0.02, outer=40, inner=3,
                        seed=BF_SEED)
    six = refrun.run_bf(os.path.join(tmp, "bf6"), c, ang, th, 0.1, 0.02, outer=4, inner=3,
                        seed=BF_SEED)
    np.savez_compressed(os.path.join(HERE, "bf_small.npz"), counts=c, tilts=ang, thickness=th,
                        object_yxz=out["object_yxz"], gain=out["gain"], offset=out["offset"],
                        variance=out["variance"], sinogram=out["sinogram"],
                        c6_object_yxz=six["object_yxz"], c6_offset=six["offset"],
                        c6_variance=six["variance"])


def haadf_cfg0(tmp):
    y, ang = cfg0_input()
    rec = {"input_counts_sha256": digest(y), "input_tilts_sha256": digest(ang),
           "shape": list(y.shape), "thickness": 32.0, "diffuseness": 0.1, "sigma_x": 0.2,
           "seed": HAADF_SEED, "runs": {}}
    for outer in (1, 5, 20):
        o = refrun.run_haadf(os.path.join(tmp, f"c0_{outer}"), y, ang, 32.0, 0.1, 0.2, outer,
                             seed=HAADF_SEED)
        rec["runs"][str(outer)] = {
            k: {"sha256": digest(o[k]), "sum": float(np.sum(o[k])),
                "norm": float(np.linalg.norm(o[k]))}
            for k in ("object_yxz", "gain", "offset", "sinogram")}
    with open(os.path.join(HERE, "haadf_cfg0.json"), "w") as f:
        json.dump(rec, f, indent=1, sort_keys=True)


def main():
    if not refrun.ensure_built():
        print("make_golden: the reference programs are not available", file=sys.stderr)
        return 1
    makers = [haadf_small, output_headers, bf_small, haadf_cfg0, haadf_bf_assist_small,
              bf_multires_small, shepp_logan]
    wanted = set(sys.argv[1:])
    with tempfile.TemporaryDirectory() as tmp:
        for make in makers:
            if not wanted or make.__name__ in wanted:
                make(tmp)
    for f in sorted(os.listdir(HERE)):
        print(f, os.path.getsize(os.path.join(HERE, f)))
    return 0


if __name__ == "__main__":
    sys.exit(main())
