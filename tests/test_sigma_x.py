"""mbir_estimate_sigma_x (host only) against the reference's SigmaXEstimation filter, run by
oracle/_ref/SigmaXEstimate (the reference built from its sources; skipped where the reference
tree is absent), on MRC tilt series of three sample modes, with the default region (read past
each row and past the last view as the reference reads it) and with explicit regions, HAADF
and bright-field (log) forms."""
import os
import subprocess
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "oracle"))

import refrun  # noqa: E402

needs_ref = pytest.mark.skipif(not refrun.ensure_built(),
                               reason="the reference tree is not present on this host")


def reference_estimate(path, thickness, gain, bf, x, y, tilts):
    exe = os.path.join(refrun.REF_DIR, "SigmaXEstimate")
    args = [exe, str(path), repr(thickness), repr(gain), "1" if bf is not None else "0",
            repr(0.0 if bf is None else bf), str(x[0]), str(x[1]), str(y[0]), str(y[1])]
    args += [repr(float(t)) for t in tilts]
    r = subprocess.run(args, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    return float(r.stdout.strip().splitlines()[-1])


def write_series(path, mode, seed):
    import synthetic
    rng = np.random.default_rng(seed)
    ang = synthetic.tilt_angles(60.0, 10.0)
    counts = rng.uniform(50, 3000, (len(ang), 40, 12))
    synthetic.write_tilt_series_mrc(str(path), counts, ang, mode=mode)
    return ang


@needs_ref
@pytest.mark.parametrize("mode", [1, 2, 6])
@pytest.mark.parametrize("bf", [None, 5.0])
@pytest.mark.parametrize("region", ["default", "box"])
def test_sigma_x_estimate_matches_reference(lib_built, tmp_path, mode, bf, region):
    mbir = lib_built
    ang = write_series(tmp_path / "s.mrc", mode, seed=mode)
    x, y = ((-1, -1), (-1, -1)) if region == "default" else ((3, 30), (2, 9))
    ref = reference_estimate(tmp_path / "s.mrc", 64.0, 1.5, bf, x, y, ang)
    got = mbir.estimate_sigma_x(tmp_path / "s.mrc", 64.0, 1.5, bf_offset=bf, tilts=ang,
                                x_range=x, y_range=y)
    assert got == ref, (got, ref)


def test_sigma_x_estimate_header_tilts(lib_built, tmp_path):
    """Without tilts the estimate takes the FEI header's a-tilts."""
    mbir = lib_built
    ang = write_series(tmp_path / "s.mrc", 2, seed=4)
    a = mbir.estimate_sigma_x(tmp_path / "s.mrc", 32.0)
    b = mbir.estimate_sigma_x(tmp_path / "s.mrc", 32.0, tilts=ang)
    assert a == b and a > 0
