"""Run OpenMBIR-TEM's own reconstruction programs on synthetic inputs, and map their
parameters onto the CPU restatement.

TEST INFRASTRUCTURE ONLY: used by tests/test_oracle_vs_ref.py and tests/golden/make_golden.py
to pin oracle/mbir_oracle.c to outputs of the reference itself.  The programs are the
reference's HAADFReconstruction and BFReconstruction built from their own sources by
oracle/build_ref.py into oracle/_ref/ (present only where the reference tree is).

What a reference run depends on, besides the algorithm:

* pixel size: the reference takes delta_r = delta_t = (float pixel size from the FEI extended
  header) * 1e9 (MRCSinogramInitializer.cpp:214-215), so a header value of 1e-9 m gives
  0.99999997171... nm, not 1 nm (REF_DELTA below);
* float parameters: the multi-resolution pipeline keeps thickness, target gain, stop threshold,
  sigma_x, diffuseness, default offset / variance / reconstruction value and the Bragg T, delta
  and offset as `float` members (HAADF_MultiResolutionReconstruction.h:76-89,
  BFMultiResolutionReconstruction.h:76-107); p = diffuseness + 1 is evaluated in float
  (HAADF_MultiResolutionReconstruction.cpp:333) and sigma_x of level i is
  2^((L-1-i)(1-3/p)) * float(sigma_x) (:340);
* visit orders: every generator is seeded from the millisecond clock.  Runs here set
  MBIR_REF_FIXED_MS, so every generator starts from that one seed (oracle: orc_run with that
  seed; orc_bf_run_fixed_seed);
* one worker (MBIR_REF_THREADS=1): the y range is one task, the sequential ICD;
* the bright-field pipeline always extends the object (BFMultiResolutionReconstruction.cpp:76,
  the command line never sets it), and its default offset is float(-log(dosage + bf_offset))
  (BFReconstructionArgsParser.cpp:272-274).
"""
import os
import shutil
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
HAADF_EXE = os.path.join(REF_DIR, "HAADFReconstruction")
BF_EXE = os.path.join(REF_DIR, "BFReconstruction")
REF_DELTA = float(np.float32(1e-9)) * 1.0e9
DEFAULT_REFERENCE = "/root/reference"

if HERE not in sys.path:
    sys.path.insert(0, HERE)
import oracle as _oracle  # noqa: E402


def f32(v):
    return float(np.float32(v))


def ensure_built(reference=DEFAULT_REFERENCE):
    """Build oracle/_ref when the reference tree is present; True when both programs exist."""
    if os.path.isdir(os.path.join(reference, "Code", "MBIRLib")):
        import build_ref
        build_ref.build(reference, quiet=True)
    return os.path.exists(HAADF_EXE) and os.path.exists(BF_EXE)


def write_mrc(path, counts_trt, tilts_deg):
    """The tilt series as the reference reads it: MRC float32, FEI extended header with
    a_tilt and a 1e-9 m pixel size."""
    pkg = os.path.join(os.path.dirname(HERE), "openmbir-tem_gb300")
    if pkg not in sys.path:
        sys.path.insert(0, pkg)
    import synthetic
    synthetic.write_tilt_series_mrc(path, np.asarray(counts_trt, np.float32), tilts_deg)


def haadf_params(thickness, diffuseness, sigma_x, outer, inner=1, stop=0.0, target_gain=1.0,
                 default_offset=0.0, use_default_offset=False, default_variance=1.0,
                 default_recon=0.0, extend_object=False, levels=1, level=None, final_res=1,
                 pinned_pow=False):
    """The oracle parameters the HAADF pipeline gives its engine for resolution level
    `level` (default: the finest), HAADF_MultiResolutionReconstruction.cpp:315-360."""
    o = _oracle.OrcParams()
    lvl = levels - 1 if level is None else level
    o.delta_xz_factor = 2.0 ** (levels - 1 - lvl) * final_res
    o.interpolate_factor = 2.0 ** (levels - 1) * final_res
    o.length_z = f32(thickness)
    o.extend_object = int(extend_object)
    o.x_shrink_factor = 0.6
    o.z_stretch = 2
    o.response_bins = 64
    o.profile_resolution = 1536
    o.beam_resolution = 512
    o.compat_double_angle = 1
    q = float(np.float32(np.float32(diffuseness) + np.float32(1.0)))
    o.sigma_x = 2.0 ** ((levels - 1 - lvl) * (1 - 3 / q)) * f32(sigma_x)
    o.mrf_p = 2.0
    o.mrf_q = q
    o.mrf_c = 0.001
    o.mrf_alpha = 1.5
    o.target_gain = f32(target_gain)
    o.default_offset = f32(default_offset)
    o.default_variance = f32(default_variance)
    o.default_recon_value = f32(default_recon)
    o.use_default_offset = int(use_default_offset)
    o.joint_estimation = 1
    o.noise_model = 1
    o.zero_skipping = 1
    o.stop_threshold = f32(stop) * (2.0 if lvl >= 2 else 1.0)
    o.outer_iterations = outer
    o.inner_iterations = inner if lvl == 0 else 1
    o.threshold_reduction_factor = 1.0
    o.pinned_pow = int(pinned_pow)
    o.modality = 0
    return o


def bf_params(thickness, diffuseness, sigma_x, outer, inner=1, stop=0.0, target_gain=1.0,
              dosage=1.0e4, use_default_dosage=True, bf_offset=0.0, default_variance=1.0,
              default_recon=0.0, bragg_t=3.0, bragg_delta=0.5, levels=1, level=None,
              final_res=1, pinned_pow=False):
    """The oracle parameters the BF pipeline gives its engine (BFMultiResolutionReconstruction
    .cpp and BFReconstructionArgsParser.cpp:255-285)."""
    o = haadf_params(thickness, diffuseness, sigma_x, outer, inner, stop, target_gain,
                     0.0, use_default_dosage, default_variance, default_recon, True, levels,
                     level, final_res, pinned_pow)
    o.default_offset = f32(-np.log(dosage + bf_offset)) if use_default_dosage else 0.0
    o.compat_double_angle = 0
    o.mrf_c = 0.01
    o.noise_model = 0
    o.modality = 1
    o.noise_estimation = 1
    o.bragg_threshold = f32(bragg_t)
    o.bragg_delta = f32(bragg_delta)
    o.bf_offset = f32(bf_offset)
    o.nhicd = 1
    return o


def _run(exe, args, workdir, seed, threads, timeout):
    env = dict(os.environ)
    env["MBIR_REF_FIXED_MS"] = str(int(seed))
    env["MBIR_REF_THREADS"] = str(int(threads))
    r = subprocess.run([exe] + args, cwd=workdir, env=env, capture_output=True, text=True,
                       timeout=timeout)
    with open(os.path.join(workdir, "log.txt"), "w") as f:
        f.write(r.stdout + r.stderr)
    if r.returncode != 0:
        raise RuntimeError(f"{os.path.basename(exe)} exited {r.returncode}: {r.stdout[-2000:]}")


def run_haadf(workdir, counts, tilts, thickness, diffuseness, sigma_x, outer, inner=1,
              stop=0.0, target_gain=1.0, seed=12345, threads=1, initial=None, levels=1,
              subvolume=None, extra=(), timeout=1800, brightfield=None):
    """Run HAADFReconstruction on counts[theta][r][t]; returns the finest level's outputs.
    `initial`: starting volume [y][x][z] (the --initial_recon_file layout); `brightfield`:
    bright-field counts of the same size (--brightfield)."""
    if os.path.exists(workdir):
        shutil.rmtree(workdir)
    os.makedirs(workdir)
    n_theta, n_r, n_t = counts.shape
    write_mrc(os.path.join(workdir, "in.mrc"), counts, tilts)
    sv = subvolume or (0, 0, 0, n_r - 1, n_t - 1, n_theta - 1)
    args = ["--sinofile", "in.mrc", "--outputfile", os.path.join(workdir, "out", "recon.mrc"),
            "--subvolume", ",".join(str(v) for v in sv), "--thickness", repr(thickness),
            "--diffuseness", repr(diffuseness), "--sigma_x", repr(sigma_x),
            "--num_resolutions", str(levels), "--outer_iterations", str(outer),
            "--inner_iterations", str(inner), "--stop_threshold", repr(stop),
            "--target_gain", repr(target_gain)] + list(extra)
    if initial is not None:
        np.ascontiguousarray(initial, "<f8").tofile(os.path.join(workdir, "init.bin"))
        args += ["--initial_recon_file", os.path.join(workdir, "init.bin")]
    if brightfield is not None:
        write_mrc(os.path.join(workdir, "bf.mrc"), brightfield, tilts)
        args += ["--brightfield", os.path.join(workdir, "bf.mrc")]
    _run(HAADF_EXE, args, workdir, seed, threads, timeout)
    return read_outputs(os.path.join(workdir, "out", "1x"), n_theta, n_r, n_t)


def run_bf(workdir, counts, tilts, thickness, diffuseness, sigma_x, outer, inner=1, stop=0.0,
           dosage=1.0e4, bragg_t=3.0, bragg_delta=0.5, seed=777, threads=1, levels=1,
           subvolume=None, extra=(), timeout=1800):
    """Run BFReconstruction on raw counts[theta][r][t]; returns the finest level's outputs."""
    if os.path.exists(workdir):
        shutil.rmtree(workdir)
    os.makedirs(workdir)
    n_theta, n_r, n_t = counts.shape
    write_mrc(os.path.join(workdir, "in.mrc"), counts, tilts)
    sv = subvolume or (0, 0, 0, n_r - 1, n_t - 1, n_theta - 1)
    args = ["--sinofile", "in.mrc", "--outputfile", os.path.join(workdir, "out", "recon.mrc"),
            "--subvolume", ",".join(str(v) for v in sv), "--thickness", repr(thickness),
            "--diffuseness", repr(diffuseness), "--sigma_x", repr(sigma_x),
            "--num_resolutions", str(levels), "--outer_iterations", str(outer),
            "--inner_iterations", str(inner), "--stop_threshold", repr(stop),
            "--target_gain", "1", "--default_dosage", repr(dosage), "--use_default_dosage",
            "--bragg_T", repr(bragg_t), "--bragg_delta", repr(bragg_delta)] + list(extra)
    _run(BF_EXE, args, workdir, seed, threads, timeout)
    return read_outputs(os.path.join(workdir, "out", "1x"), n_theta, n_r, n_t)


def read_outputs(d, n_theta, n_r, n_t):
    """The level's output files as arrays: volume [z][x][y] (from ReconstructedObject.bin, written
    y-x-z by RawGeometryWriter.cpp:83-91), gain/offset/variance per view, and the final sinogram
    (counts - e) * I + mu (SinogramBinWriter.cpp:115-126)."""
    out = {}
    obj = np.fromfile(os.path.join(d, "ReconstructedObject.bin"), "<f8")
    for name, key in (("FinalGainParameters.bin", "gain"), ("FinalOffsetParameters.bin", "offset"),
                      ("FinalVariances.bin", "variance")):
        p = os.path.join(d, name)
        if os.path.exists(p):
            out[key] = np.fromfile(p, "<f8")
    sino = os.path.join(d, "ReconstructedSinogram.bin")
    if os.path.exists(sino):
        out["sinogram"] = np.fromfile(sino, "<f8").reshape(n_theta, n_r, n_t)
    out["object_yxz"] = obj
    return out


def volume_zxy(out, n_z, n_x, n_y):
    """ReconstructedObject.bin (y-x-z) as [z][x][y]."""
    return np.ascontiguousarray(np.transpose(out["object_yxz"].reshape(n_y, n_x, n_z), (2, 1, 0)))


def oracle_sinogram(orc, counts):
    """The oracle's counterpart of ReconstructedSinogram.bin."""
    return ((np.asarray(counts, np.float64) - orc.error()) * orc.gain()[:, None, None]
            + orc.offset()[:, None, None])
