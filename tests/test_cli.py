"""The command-line programs bin/HAADFReconstruction and bin/BFReconstruction (the reference's
flag sets over the C ABI).

CPU: flag parsing (unknown flags, missing required flags and values fail with exit status 1,
as the reference's TCLAP parser does; --help succeeds).  GPU: a reconstruction from an MRC tilt
series writes the reference's output files, with the headers of the reference's own MRC, VTK
and Avizo files for the same case (tests/golden/output_headers.json, written by the reference
itself), and the same volume as the library run with the same parameters.
"""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
BIN = os.path.join(ROOT, "openmbir-tem_gb300", "bin")
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def run(prog, *args, cwd=None):
    exe = os.path.join(BIN, prog)
    return subprocess.run([exe] + list(args), capture_output=True, text=True, cwd=cwd,
                          timeout=600)


@pytest.fixture(scope="module")
def cli_built(lib_built):
    assert os.path.exists(os.path.join(BIN, "HAADFReconstruction"))
    assert os.path.exists(os.path.join(BIN, "BFReconstruction"))
    return True


def test_cli_unknown_flag_fails(cli_built):
    r = run("HAADFReconstruction", "--sinofile", "x.mrc", "--bogus", "1")
    assert r.returncode == 1
    assert "Couldn't find match for argument" in r.stdout


def test_cli_missing_required_flag_fails(cli_built):
    r = run("HAADFReconstruction", "--sinofile", "x.mrc", "--outputfile", "o/r.mrc",
            "--thickness", "16")
    assert r.returncode == 1 and "Required argument missing" in r.stdout
    r = run("BFReconstruction", "--sinofile", "x.mrc", "--outputfile", "o/r.mrc",
            "--thickness", "16", "--sigma_x", "0.02", "--subvolume", "0,0,0,63,7,30")
    assert r.returncode == 1 and "default_dosage" in r.stdout


def test_cli_missing_value_and_bad_subvolume_fail(cli_built):
    r = run("HAADFReconstruction", "--sinofile")
    assert r.returncode == 1 and "Missing a value" in r.stdout
    r = run("HAADFReconstruction", "-s", "x.mrc", "--outputfile", "o/r.mrc", "--thickness", "16",
            "--sigma_x", "0.2", "--target_gain", "1", "--subvolume", "1,2,3")
    assert r.returncode == 1 and "Subvolume" in r.stdout


def test_cli_help(cli_built):
    r = run("BFReconstruction", "--help")
    assert r.returncode == 0 and "--bragg_T" in r.stdout and "--default_dosage" in r.stdout


@pytest.mark.gpu
def test_cli_haadf_reconstruction_files(cli_built, tmp_path):
    import mbir
    import refrun
    from conftest import small_case
    y, ang, th = small_case()
    refrun.write_mrc(str(tmp_path / "in.mrc"), y, ang)
    out = tmp_path / "out"
    # the whole series as the subvolume, as the run that wrote the header fixture had it (without
    # the flag the reference hands its engine six zeros, a 63 x 3 detector window of one view)
    n_theta, n_r, n_t = y.shape
    sv = (0, 0, 0, n_r - 1, n_t - 1, n_theta - 1)
    r = run("HAADFReconstruction", "-s", str(tmp_path / "in.mrc"), "--outputfile",
            str(out / "recon.mrc"), "--subvolume", ",".join(str(v) for v in sv), "--thickness",
            "16", "--diffuseness", "0.1", "--sigma_x", "0.2", "--num_resolutions", "1",
            "--outer_iterations", "1", "--inner_iterations", "1", "--stop_threshold", "0",
            "--target_gain", "1")
    assert r.returncode == 0, r.stdout + r.stderr
    with open(os.path.join(HERE, "golden", "output_headers.json")) as f:
        ref = json.load(f)
    mrc = (out / "recon.mrc").read_bytes()
    rh = bytes.fromhex(ref["mrc_header_hex"])
    assert len(mrc) == ref["mrc_size"]
    # every header byte but the value range and mean (bytes 76-87) equals the reference's
    assert mrc[:76] == rh[:76] and mrc[88:1024] == rh[88:1024]
    n_ext = int.from_bytes(mrc[92:96], "little")
    assert mrc[1024:1024 + n_ext] == bytes.fromhex(ref["mrc_ext_header_hex"])
    vtk = (out / "recon.vtk").read_bytes()
    assert len(vtk) == ref["vtk_size"] and vtk.startswith(ref["vtk_header"].encode())
    am = (out / "recon.am").read_bytes()
    assert len(am) == ref["am_size"] and am.startswith(ref["am_header"].encode())
    for name in ("ReconstructedObject.bin", "FinalGainParameters.bin",
                 "FinalOffsetParameters.bin", "FinalVariances.bin", "ReconstructedSinogram.bin",
                 "0_0_ReconstructedVolume.rec"):
        assert (out / "1x" / name).exists(), name
    # the intermediate image of the one outer iteration is the final volume in the same format
    rec = (out / "1x" / "0_0_ReconstructedVolume.rec").read_bytes()
    assert len(rec) == len(mrc) and rec[1024:] == mrc[1024:]
    # the same run through the library: the command line maps its flags onto these parameters
    p = mbir.default_params()
    p.sample_thickness = 16.0
    p.diffuseness = 0.1
    p.sigma_x = 0.2
    p.num_resolutions = 1
    p.outer_iterations = 1
    p.inner_iterations = 1
    p.stop_threshold = 0.0
    p.target_gain = 1.0
    p.float_params = 1
    p.use_subvolume = 1
    for i, v in enumerate(sv):
        p.subvolume[i] = v
    with mbir.Engine(p) as e:
        e.load_mrc(str(tmp_path / "in.mrc"))
        e.run()
        vol = e.volume()
        nz, nx, ny = e.dims()[:3]
    obj = np.fromfile(out / "1x" / "ReconstructedObject.bin", "<f8").reshape(ny, nx, nz)
    np.testing.assert_array_equal(np.transpose(obj, (2, 1, 0)), vol.astype(np.float64))


@pytest.mark.gpu
def test_cli_bf_two_levels(cli_built, tmp_path):
    """Two resolution levels of bright field: level directories 2x and 1x, the final volume at
    the fine level's size (the object extended in x, as the reference's BF pipeline does)."""
    import refrun
    from conftest import bf_case
    c, ang, th = bf_case()
    refrun.write_mrc(str(tmp_path / "in.mrc"), c, ang)
    out = tmp_path / "out"
    n_theta, n_r, n_t = c.shape
    r = run("BFReconstruction", "-s", str(tmp_path / "in.mrc"), "--outputfile",
            str(out / "recon.mrc"), "--subvolume", f"0,0,0,{n_r - 1},{n_t - 1},{n_theta - 1}",
            "--thickness", "16", "--diffuseness", "0.1", "--sigma_x", "0.02",
            "--num_resolutions", "2", "--outer_iterations", "4", "--inner_iterations", "2",
            "--stop_threshold", "0", "--default_dosage", "10000", "--use_default_dosage")
    assert r.returncode == 0, r.stdout + r.stderr
    for lvl in ("2x", "1x"):
        assert (out / lvl / "ReconstructedObject.bin").exists(), lvl
    assert (out / "recon.mrc").exists() and (out / "recon.vtk").exists()
    fine = np.fromfile(out / "1x" / "ReconstructedObject.bin", "<f8")
    coarse = np.fromfile(out / "2x" / "ReconstructedObject.bin", "<f8")
    assert fine.size == 8 * coarse.size
    assert np.all(np.isfinite(fine)) and fine.max() > 0


@pytest.mark.gpu
def test_cli_haadf_with_bright_field(cli_built, tmp_path):
    """--brightfield: the bright-field tilt series read with the sinogram's subvolume; the same
    volume as the library run with the same files."""
    import mbir
    import refrun
    g = dict(np.load(os.path.join(HERE, "golden", "haadf_bf_assist_small.npz")))
    y, bf, ang = g["counts"], g["bf_counts"], g["tilts"]
    refrun.write_mrc(str(tmp_path / "in.mrc"), y, ang)
    refrun.write_mrc(str(tmp_path / "bf.mrc"), bf, ang)
    n_theta, n_r, n_t = y.shape
    sv = (0, 0, 0, n_r - 1, n_t - 1, n_theta - 1)
    out = tmp_path / "out"
    r = run("HAADFReconstruction", "-s", str(tmp_path / "in.mrc"), "--brightfield",
            str(tmp_path / "bf.mrc"), "--outputfile", str(out / "recon.mrc"), "--subvolume",
            ",".join(str(v) for v in sv), "--thickness", "16", "--diffuseness", "0.1",
            "--sigma_x", "0.2", "--num_resolutions", "1", "--outer_iterations", "2",
            "--inner_iterations", "1", "--stop_threshold", "0", "--target_gain", "1")
    assert r.returncode == 0, r.stdout + r.stderr
    p = mbir.default_params()
    p.sample_thickness = 16.0
    p.diffuseness = 0.1
    p.sigma_x = 0.2
    p.num_resolutions = 1
    p.outer_iterations = 2
    p.inner_iterations = 1
    p.stop_threshold = 0.0
    p.target_gain = 1.0
    p.float_params = 1
    p.use_subvolume = 1
    for i, v in enumerate(sv):
        p.subvolume[i] = v
    with mbir.Engine(p) as e:
        e.load_mrc(str(tmp_path / "in.mrc"))
        e.load_bright_field_mrc(str(tmp_path / "bf.mrc"))
        e.run()
        vol = e.volume()
        nz, nx, ny = e.dims()[:3]
    obj = np.fromfile(out / "1x" / "ReconstructedObject.bin", "<f8").reshape(ny, nx, nz)
    np.testing.assert_array_equal(np.transpose(obj, (2, 1, 0)), vol.astype(np.float64))
