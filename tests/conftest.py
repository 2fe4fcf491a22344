import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "openmbir-tem_gb300")
ORACLE = os.path.join(ROOT, "oracle")
for p in (PKG, ORACLE, os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def has_gpu():
    try:
        import torch  # noqa: F401  (plumbing only: device query)
        return torch.cuda.is_available()
    except Exception:
        return False


def pytest_collection_modifyitems(config, items):
    if has_gpu():
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


@pytest.fixture(scope="session")
def lib_built():
    import build as pkg_build
    pkg_build.build()
    import mbir
    return mbir


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.build()
    return oracle


def small_case(n_r=64, n_t=8, max_deg=70.0, step=4.0, seed=3, thickness=16.0):
    """A reduced two-sphere HAADF case that the FP64 oracle sweeps in well under a second."""
    import synthetic
    ang = synthetic.tilt_angles(max_deg, step)
    shapes = [(-12.0, 0.0, 0.0, 10.0, 10.0, 10.0, 1.0), (15.0, 1.0, 3.0, 6.0, 6.0, 6.0, 0.5)]
    proj = synthetic.ellipsoid_projection(ang, n_r, n_t, shapes)
    y, _ = synthetic.haadf_measurements(proj, seed=seed)
    return y, ang.astype(np.float32), thickness


def haadf_params(mbir, thickness, **kw):
    p = mbir.default_params()
    p.sample_thickness = thickness
    p.diffuseness = 0.1
    p.sigma_x = 0.2
    p.num_resolutions = 1
    p.outer_iterations = 5
    p.inner_iterations = 1
    p.stop_threshold = 0.0
    p.lane_shape = 1  # fixed voxel-group shape: engines compared bit for bit must agree
    p.seed_mode = mbir.SEED_FIXED  # reference order: one visit order for every sweep
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def bf_case(n_r=64, n_t=8, max_deg=60.0, step=4.0, seed=2, thickness=16.0, n_particles=6):
    """A reduced bright-field case: a few ellipsoids seen as Poisson counts (1e4 electrons,
    +-3% per-view dose drift).  Returns (counts, angles, thickness)."""
    import synthetic
    ang = synthetic.tilt_angles(max_deg, step)
    shapes = synthetic.random_ellipsoids(n_particles, n_r, n_t, 2 * thickness, seed=seed,
                                         axes=(3.0, 8.0), z_range=(-thickness / 4, thickness))
    proj = synthetic.ellipsoid_projection(ang, n_r, n_t, shapes)
    counts, _ = synthetic.bf_counts(proj, seed=seed + 1)
    return counts, ang.astype(np.float32), thickness


def bf_params(mbir, thickness, **kw):
    p = mbir.default_params(mbir.BF)
    p.sample_thickness = thickness
    p.diffuseness = 0.1
    p.sigma_x = 0.02
    p.num_resolutions = 1
    p.outer_iterations = 5
    p.inner_iterations = 1
    p.stop_threshold = 0.0
    p.use_default_offset = 1
    p.default_dosage = 1.0e4
    p.bragg_threshold = 3.0
    p.lane_shape = 1
    for k, v in kw.items():
        setattr(p, k, v)
    return p
