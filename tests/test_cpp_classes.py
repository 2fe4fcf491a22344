"""The C++ classes of include/mbir_gb300.hpp (HAADF_ReconstructionEngine, BFReconstructionEngine,
HAADF_MultiResolutionReconstruction, BFMultiResolutionReconstruction over the C ABI), through
the test program tests/cpp/compat_classes.cpp.

CPU: the header compiles and links against the library; error conditions without a GPU (an
engine with no sinogram, results read before a load, an output directory that cannot be made, a
cancel set before execute() gives the reference's -999); the pipeline's per-level parameters.  GPU: an engine run from arrays gives
the same volume, bit for bit, as the C ABI run with the same parameters, twice on the same
object, with the observer seeing each run complete; setCancel(true) from another thread ends a
long run with -999.  The pipeline classes' GPU runs are the command-line programs' tests
(tests/test_cli.py), which are built on them.
"""
import os
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
PKG = os.path.join(ROOT, "openmbir-tem_gb300")

MBIR_EDEVICE, MBIR_EIO, MBIR_ESTATE, MBIR_ECANCELLED = -3, -4, -5, -999


@pytest.fixture(scope="module")
def compat_exe(lib_built, tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("cpp") / "compat_classes")
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror", "-pthread",
           "-I", os.path.join(ROOT, "include"), "-o", exe,
           os.path.join(HERE, "cpp", "compat_classes.cpp"), f"-L{PKG}", "-l:libmbir_gb300.so",
           f"-Wl,-rpath,{PKG}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return exe


def run(exe, *args):
    r = subprocess.run([exe] + [str(a) for a in args], capture_output=True, text=True,
                       timeout=600)
    out = {}
    for line in r.stdout.splitlines():
        k, *v = line.split()
        out[k] = [float(x) if k.endswith("_f") else int(x) for x in v]
    return r, out


def test_classes_error_paths(compat_exe, tmp_path):
    r, out = run(compat_exe, "errors", tmp_path)
    assert r.returncode == 0, r.stdout + r.stderr
    assert out["volume_before_load"] == [MBIR_ESTATE]
    rc, cond, has_msg = out["no_sinogram"]
    # no GPU: the engine cannot be created; with one: there is no sinogram to read
    assert rc in (MBIR_EDEVICE, MBIR_ESTATE) and cond == rc and has_msg == 1
    assert out["output_dir"] == [MBIR_EIO, MBIR_EIO, 1]
    assert out["cancel_before"] == [MBIR_ECANCELLED, 1]


def test_pipeline_level_parameters(compat_exe):
    """The per-level rules of HAADF_MultiResolutionReconstruction.cpp:318-357 for three levels:
    voxels of 2^(L-1-i) * final_resolution pixels, p = diffuseness + 1 in float, sigma_x scaled
    by 2^((L-1-i)(1-3/p)), the inner iterations and the default volume, variance and offset on
    the first level only, the stop threshold doubled (in float) from the third level, the
    previous level's volume interpolated from the second level."""
    r, out = run(compat_exe, "levels")
    assert r.returncode == 0, r.stdout + r.stderr
    L = 3
    f32 = np.float32
    p = float(f32(0.2) + f32(1.0))
    for i in range(L):
        level, factor, inner, outer, use_off, interp, float_params = out[f"level{i}"]
        assert (level, factor, outer, float_params) == (i, 2 ** (L - 1 - i) * 2, 7, 1)
        assert inner == (10 if i == 0 else 1)
        assert use_off == (1 if i == 0 else 0) and interp == (0 if i == 0 else 1)
        sigma, q, stop, recon, var, off = out[f"level{i}_f"]
        assert q == p
        assert sigma == 2.0 ** ((L - 1 - i) * (1 - 3 / p)) * float(f32(0.3))
        assert stop == (float(f32(0.005) * f32(2.0)) if i >= 2 else 0.005)
        assert (recon, var, off) == ((0.5, 2.0, 0.1) if i == 0 else (0.0, 1.0, 0.0))


def small_inputs(tmp_path):
    from conftest import small_case
    y, ang, th = small_case()
    n_theta, n_r, n_t = y.shape
    y.astype(np.float32).tofile(tmp_path / "counts.f32")
    ang.astype(np.float32).tofile(tmp_path / "tilts.f32")
    return y, ang, th, (n_theta, n_r, n_t)


@pytest.mark.gpu
def test_engine_class_matches_c_abi(compat_exe, tmp_path):
    import mbir
    from conftest import haadf_params
    y, ang, th, shape = small_inputs(tmp_path)
    r, out = run(compat_exe, "run", tmp_path / "counts.f32", tmp_path / "tilts.f32", *shape, th,
                 tmp_path / "vol.f32")
    assert r.returncode == 0, r.stdout + r.stderr
    assert out["execute"] == [0] and out["execute_again"] == [0]
    assert out["nuisance"] == [0, shape[0]]
    assert out["same_volume"] == [1]
    assert out["complete"] == [2]  # the observer, registered at each load
    p = haadf_params(mbir, th)
    with mbir.Engine(p) as e:
        e.set_sinogram(y, ang)
        e.run()
        vol = e.volume()
        dims = e.dims()
    assert out["dims"] == [int(v) for v in dims]
    got = np.fromfile(tmp_path / "vol.f32", np.float32).reshape(vol.shape)
    np.testing.assert_array_equal(got, vol)


@pytest.mark.gpu
def test_engine_class_cancel_from_another_thread(compat_exe, tmp_path):
    y, ang, th, shape = small_inputs(tmp_path)
    r, out = run(compat_exe, "cancel", tmp_path / "counts.f32", tmp_path / "tilts.f32", *shape,
                 th)
    assert r.returncode == 0, r.stdout + r.stderr
    assert out["cancel"] == [MBIR_ECANCELLED, MBIR_ECANCELLED, 1]
