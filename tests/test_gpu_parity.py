"""GPU parity: the sm_103a engine, called through the C ABI, against the FP64 oracle.

Tolerances (FP32 volume / error sinogram / footprints on the GPU, FP64 oracle):
  forward projection of a fixed volume      max|dy| / max|y|         <= 1e-5
  one ICD sweep in the same visit order     ||dx|| / ||x||           <= 1e-5
  reference-order iterates after 5 outer    ||dx|| / ||x||           <= 1e-4
  gain/offset/variance estimates            relative                 <= 1e-6 (same inputs)
  converged volume, parallel vs reference   ||dx|| / ||x||           <= 1e-3
"""
import os

import numpy as np
import pytest

from conftest import haadf_params, small_case

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-300))


def pair(mbir, oracle_mod, case=None, **kw):
    y, ang, th = case if case is not None else small_case()
    p = haadf_params(mbir, th, **kw)
    e = mbir.Engine(p)
    e.set_sinogram(y, ang)
    o = oracle_mod.Oracle(oracle_mod.params_from_mbir(p), y, ang)
    return e, o, p, y


def test_forward_projection_matches_oracle(lib_built, oracle_mod):
    e, o, p, y = pair(lib_built, oracle_mod)
    nz, nx, ny = e.dims()[:3]
    vol = np.random.default_rng(1).random((nz, nx, ny)).astype(np.float32)
    e.set_initial_volume(vol)
    e.prepare()
    o.prepare(vol.astype(np.float64))
    yg, yo = e.projection(), o.yest()
    err = np.abs(yg - yo).max() / np.abs(yo).max()
    assert err <= 1e-5, err
    eg, eo = e.error_sinogram(), o.error()
    assert np.abs(eg - eo).max() / np.abs(y).max() <= 1e-5


def test_forward_projection_two_spheres_full_size(lib_built, oracle_mod):
    """The 128x32x64 HAADF case: projection of the voxelised two-sphere phantom."""
    import synthetic
    y, ang, _ = synthetic.haadf_two_spheres()
    e, o, p, y = pair(lib_built, oracle_mod, case=(y, ang, 32.0))
    nz, nx, ny = e.dims()[:3]
    z = -nz / 2 + np.arange(nz) + 0.5
    x = -nx / 2 + np.arange(nx) + 0.5
    yy = -ny / 2 + np.arange(ny) + 0.5
    Z, X, Y = np.meshgrid(z, x, yy, indexing="ij")
    vol = np.zeros((nz, nx, ny), np.float32)
    for (cx, cy, cz, ax, ay, az, val) in synthetic.two_sphere_shapes():
        vol += val * ((((X - cx) / ax) ** 2 + ((Y - cy) / ay) ** 2 + ((Z - cz) / az) ** 2) <= 1)
    e.set_initial_volume(vol)
    e.prepare()
    o.prepare(vol.astype(np.float64))
    err = np.abs(e.projection() - o.yest()).max() / np.abs(o.yest()).max()
    assert err <= 1e-5, err


def test_parallel_sweep_fp32_matches_oracle_same_order(lib_built, oracle_mod):
    """One FP32 sweep in the engine's parallel order against the FP64 oracle in the same order.
    (Later FP32 sweeps drift from FP64 by the chaotic sensitivity of ICD iterates to rounding;
    the FP64 engine is compared over several sweeps below.)"""
    e, o, p, y = pair(lib_built, oracle_mod)
    e.prepare()
    o.prepare()
    rows, stride = e.schedule(0)
    sg = e.sweep(0, 0)
    so = o.sweep_slices(rows, stride, 0, 0)
    assert sg[3] == so[3] and sg[2] == so[2], (sg, so)  # updated / zero-skipped counts
    assert rel(e.volume(), o.volume()) <= 1e-5
    assert rel(e.error_sinogram(), o.error()) <= 1e-5


def test_parallel_sweeps_fp64_match_oracle_same_order(lib_built, oracle_mod):
    """FP64 engine, parallel order, two sweeps against the oracle in the same order.  This path
    sums theta with warp shuffles (not in the reference's order), so later sweeps may flip a
    zero-skip decision on last-bit differences; the reference-exact mode is checked below."""
    e, o, p, y = pair(lib_built, oracle_mod, precision=lib_built.FP64)
    e.prepare()
    o.prepare()
    for k in range(2):
        rows, stride = e.schedule(k)
        sg = e.sweep(0, k)
        so = o.sweep_slices(rows, stride, 0, k)
        assert sg[3] == so[3] and sg[2] == so[2], (k, sg, so)
        # FP64 state with a different summation order: the gap grows from ~1e-8 by sweep
        assert rel(e.volume(), o.volume()) <= 1e-6, (k, rel(e.volume(), o.volume()))
    e.joint_estimation()
    o.joint_estimation()
    np.testing.assert_allclose(e.nuisance()[0], o.gain(), rtol=1e-6)


def test_reference_order_iterates_after_five_outer(lib_built, oracle_mod):
    """Reference-order mode (same MT19937 visit order, one task over all y, FP64 as the
    reference's Real_t, every operation in the reference's order) reproduces the reference
    iterates after 5 outer iterations with gain/offset and variance updates."""
    e, o, p, y = pair(lib_built, oracle_mod, order_mode=1, seed=20121, outer_iterations=5,
                      precision=lib_built.FP64)
    e.run()
    o.prepare()
    n, _ = o.run(20121)
    assert n == 5 and e.status().sweeps_done == 5
    r = rel(e.volume(), o.volume())
    assert r <= 1e-4, r
    g, off, var = e.nuisance()
    assert rel(g, o.gain()) <= 1e-4
    assert rel(off, o.offset()) <= 1e-4
    assert rel(var, o.variance()) <= 1e-4


def test_reference_order_fp32_first_sweep(lib_built, oracle_mod):
    e, o, p, y = pair(lib_built, oracle_mod, order_mode=1, seed=77)
    e.prepare()
    o.prepare()
    e.sweep(0, 0)
    o.sweep_reference(77, 0, 0)
    assert rel(e.volume(), o.volume()) <= 1e-5


def test_fp32_vs_fp64_engine_precision(lib_built, oracle_mod):
    """Precision study: the FP32 engine against the all-FP64 engine from the same start, one
    sweep in the same order (error stated against the FP64 run)."""
    mbir = lib_built
    y, ang, th = small_case()
    vols = []
    for prec in (mbir.FP32, mbir.FP64):
        with mbir.Engine(haadf_params(mbir, th, precision=prec)) as e:
            e.set_sinogram(y, ang)
            e.prepare()
            e.sweep(0, 0)
            vols.append(e.volume())
    assert rel(vols[0], vols[1]) <= 1e-5


def _sync_oracle(e, o):
    o.volume()[...] = e.volume()
    o.error()[...] = e.error_sinogram()


def test_joint_estimation_and_variance_match(lib_built, oracle_mod):
    e, o, p, y = pair(lib_built, oracle_mod)
    e.prepare()
    o.prepare()
    e.sweep(0, 0)
    _sync_oracle(e, o)
    e.joint_estimation()
    o.joint_estimation()
    g, off, _ = e.nuisance()
    np.testing.assert_allclose(g, o.gain(), rtol=1e-6)
    np.testing.assert_allclose(off, o.offset(), rtol=1e-6, atol=1e-9)
    assert np.abs(e.error_sinogram() - o.error()).max() <= 1e-5 * np.abs(y).max()
    _sync_oracle(e, o)
    e.update_weights()
    o.update_weights()
    np.testing.assert_allclose(e.nuisance()[2], o.variance(), rtol=1e-6)


def test_cost_matches_oracle(lib_built, oracle_mod):
    e, o, p, y = pair(lib_built, oracle_mod)
    e.prepare()
    o.prepare()
    e.sweep(0, 0)
    _sync_oracle(e, o)
    cg, pg = e.cost()
    co, po = o.cost()
    np.testing.assert_allclose(pg[0], po[0], rtol=1e-9)   # data term: FP64 sums of equal inputs
    np.testing.assert_allclose(pg[1], po[1], rtol=1e-5)   # prior: FP32 |d|^(p-q), FP64 sums
    np.testing.assert_allclose(pg[2], po[2], rtol=1e-12)  # noise term
    np.testing.assert_allclose(cg, co, rtol=1e-6)


def test_parallel_cost_decreases_monotonically(lib_built, oracle_mod):
    e, o, p, y = pair(lib_built, oracle_mod)
    e.prepare()
    costs = [e.cost()[0]]
    for k in range(8):
        e.sweep(0, k)
        costs.append(e.cost()[0])
    assert all(b < a for a, b in zip(costs, costs[1:])), costs


def test_converged_parallel_matches_reference(lib_built, oracle_mod):
    """Fixed nuisance: the parallel (red/black, conflict-free) order and the reference's random
    order reach the same MAP volume."""
    e, o, p, y = pair(lib_built, oracle_mod, zero_skipping=0)
    e.prepare()
    o.prepare()
    for k in range(250):
        e.sweep(0, k)
        o.sweep_reference(7, 0, k)
    r = rel(e.volume(), o.volume())
    assert r <= 1e-3, r


def test_global_slice_path_matches_oracle(lib_built, oracle_mod):
    """A slice too large for shared memory (150 views x 384 bins) runs the same kernel with the
    slice in HBM; projection and sweep must match the oracle.  (Sweeps start from the default
    volume: from a random volume one ICD sweep is chaotic -- a 1e-15 relative change of the
    start moves the result by ~3e-7 -- so it cannot be compared at 1e-5.)"""
    import synthetic
    ang = np.linspace(-74.5, 74.5, 150)
    proj = synthetic.ellipsoid_projection(ang, 384, 4, [(0, 0, 0, 60, 60, 20, 1.0)])
    y, _ = synthetic.haadf_measurements(proj, seed=5)
    case = (y, ang.astype(np.float32), 24.0)
    e, o, p, y = pair(lib_built, oracle_mod, case=case)
    nz, nx, ny = e.dims()[:3]
    vol = np.random.default_rng(2).random((nz, nx, ny)).astype(np.float32)
    e.set_initial_volume(vol)
    e.prepare()
    assert e.status().staged == 0  # 150 x 388 floats per detector row exceed shared memory
    o.prepare(vol.astype(np.float64))
    assert np.abs(e.projection() - o.yest()).max() / np.abs(o.yest()).max() <= 1e-5
    e, o, p, y = pair(lib_built, oracle_mod, case=case)
    e.prepare()
    o.prepare()
    assert e.status().staged == 0
    rows, stride = e.schedule(0)
    e.sweep(0, 0)
    o.sweep_slices(rows, stride, 0, 0)
    assert rel(e.volume(), o.volume()) <= 1e-5


def test_deterministic(lib_built, oracle_mod):
    vols = []
    for _ in range(2):
        e, o, p, y = pair(lib_built, oracle_mod, outer_iterations=3)
        e.run()
        vols.append(e.volume())
        e.close()
    assert np.array_equal(vols[0], vols[1])


def test_multires_levels_run(lib_built):
    mbir = lib_built
    y, ang, th = small_case(n_r=64, n_t=12)
    p = haadf_params(mbir, th, num_resolutions=2, outer_iterations=2, inner_iterations=2)
    vol = mbir.run_multires(p, y, ang)
    with mbir.Engine(haadf_params(mbir, th, num_resolutions=2)) as e:
        e.set_sinogram(y, ang)
        assert vol.shape == e.dims()[:3]
    assert np.isfinite(vol).all() and vol.max() > 0


def test_write_outputs(lib_built, oracle_mod, tmp_path):
    import synthetic
    e, o, p, y = pair(lib_built, oracle_mod, outer_iterations=1)
    e.run()
    vol = e.volume()
    mrc = tmp_path / "recon.mrc"
    e.write_outputs(tmp_path, mrc)
    hdr, data = synthetic.read_mrc_volume(mrc)
    nz, nx, ny = vol.shape
    assert (hdr["nz"], hdr["ny"], hdr["nx"]) == (nz, ny, nx) and hdr["mode"] == 2
    assert hdr["label0"].startswith("Fei Company")
    # sections are written from z = N_z-1 down to 0 (MRCWriter.cpp:251)
    np.testing.assert_array_equal(data[0], vol[nz - 1].T)
    raw = np.fromfile(tmp_path / "ReconstructedObject.bin", np.float64).reshape(ny, nx, nz)
    np.testing.assert_array_equal(raw.transpose(2, 1, 0), vol.astype(np.float64))
    for f in ("FinalGainParameters.bin", "FinalOffsetParameters.bin", "FinalVariances.bin"):
        assert os.path.getsize(tmp_path / f) == 8 * y.shape[0]


def test_cancel_before_sweep(lib_built, oracle_mod):
    e, o, p, y = pair(lib_built, oracle_mod)
    e.prepare()
    e.cancel()
    with pytest.raises(lib_built.MbirError) as ei:
        e.sweep(0, 0)
    assert ei.value.code == -999


def test_reference_order_exact_five_sweeps_fixed_nuisance(lib_built, oracle_mod):
    e, o, p, y = pair(lib_built, oracle_mod, order_mode=1, seed=4242, precision=lib_built.FP64)
    e.prepare()
    o.prepare()
    assert rel(e.error_sinogram(), o.error()) <= 1e-7
    for k in range(5):
        sg = e.sweep(0, k)
        so = o.sweep_reference(4242, 0, k)
        assert sg[2] == so[2] and sg[3] == so[3], (k, sg, so)
    assert rel(e.volume(), o.volume()) <= 1e-6


@pytest.mark.parametrize("staging", [0, 1])
def test_sweep_staging_modes_match_oracle(lib_built, oracle_mod, staging):
    """The same sweep with the slice's detector rows in shared memory (0) and in HBM (1)."""
    e, o, p, y = pair(lib_built, oracle_mod, slice_staging=staging)
    e.prepare()
    assert e.status().staged == (1 if staging == 0 else 0)
    o.prepare()
    rows, stride = e.schedule(0)
    e.sweep(0, 0)
    o.sweep_slices(rows, stride, 0, 0)
    assert rel(e.volume(), o.volume()) <= 1e-5


def test_staged_and_hbm_paths_bit_identical(lib_built):
    """Shared-memory and HBM slices run the same arithmetic in the same order, so they agree
    bit for bit even from a random start, where ICD is chaotic."""
    mbir = lib_built
    y, ang, th = small_case()
    vols = []
    for staging in (0, 1):
        with mbir.Engine(haadf_params(mbir, th, slice_staging=staging)) as e:
            e.set_sinogram(y, ang)
            nz, nx, ny = e.dims()[:3]
            e.set_initial_volume(np.random.default_rng(3).random((nz, nx, ny)).astype(np.float32))
            e.prepare()
            for k in range(3):
                e.sweep(1 if k else 0, k)
            vols.append((e.volume(), e.error_sinogram()))
    assert np.array_equal(vols[0][0], vols[1][0])
    assert np.array_equal(vols[0][1], vols[1][1])


def test_many_views_in_shared_memory(lib_built, oracle_mod):
    """150 views (ten views per lane) with the slice staged in shared memory."""
    import synthetic
    ang = np.linspace(-74.5, 74.5, 150)
    proj = synthetic.ellipsoid_projection(ang, 96, 4, [(0, 0, 0, 20, 20, 8, 1.0)])
    y, _ = synthetic.haadf_measurements(proj, seed=6)
    e, o, p, y = pair(lib_built, oracle_mod, case=(y, ang.astype(np.float32), 16.0))
    e.prepare()
    assert e.status().staged == 1
    o.prepare()
    rows, stride = e.schedule(0)
    e.sweep(0, 0)
    o.sweep_slices(rows, stride, 0, 0)
    assert rel(e.volume(), o.volume()) <= 1e-5


@pytest.mark.parametrize("precision,tol", [(0, 1e-5), (1, 1e-7)])
def test_more_than_160_views(lib_built, oracle_mod, precision, tol):
    """241 views over +-60 deg at 0.5 deg: a parallel sweep with 32 lanes x 8 views on the slices
    in HBM, FP32 and FP64, against the oracle in the same order from the same state (the FP64
    volume is read out in float32), then a sweep that lowers the cost; the reference-order
    modes refuse the series."""
    import synthetic
    mbir = lib_built
    ang = synthetic.tilt_angles(60.0, 0.5)
    assert len(ang) == 241
    proj = synthetic.ellipsoid_projection(ang, 64, 4, [(0, 0, 0, 14, 14, 8, 1.0)])
    y, _ = synthetic.haadf_measurements(proj, seed=7)
    case = (y, ang.astype(np.float32), 16.0)
    e, o, p, y = pair(mbir, oracle_mod, case=case, precision=precision)
    e.prepare()
    st = e.status()
    assert st.staged == 0 and (precision == 1 or st.lane_shape == 5)
    o.prepare()
    assert rel(e.error_sinogram(), o.error()) <= 1e-5
    rows, stride = e.schedule(0)
    sg = e.sweep(0, 0)
    so = o.sweep_slices(rows, stride, 0, 0)
    assert sg[3] == so[3] and sg[2] == so[2], (sg, so)
    assert rel(e.volume(), o.volume()) <= tol, rel(e.volume(), o.volume())
    assert rel(e.error_sinogram(), o.error()) <= 1e-5
    c0 = e.cost()[0]
    e.sweep(0, 1)
    assert e.cost()[0] <= c0
    e.close()
    r = mbir.Engine(haadf_params(mbir, 16.0, order_mode=1))
    r.set_sinogram(*case[:2])
    with pytest.raises(mbir.MbirError):
        r.prepare()
    r.close()


def test_reference_exact_mode_bitwise(lib_built, oracle_mod):
    """The reference-exact mode performs the oracle's operations in the oracle's order (powers
    by the pinned method on both sides), so after 3 outer iterations with gain/offset and
    variance estimation the FP64 volumes round to the same float32 values."""
    e, o, p, y = pair(lib_built, oracle_mod, order_mode=1, seed=9001, outer_iterations=3,
                      precision=lib_built.FP64)
    e.run()
    o.prepare()
    o.run(9001)
    v = o.volume()
    assert np.array_equal(e.volume(), v.astype(np.float32)), rel(e.volume(), v)
    g, off, var = e.nuisance()
    np.testing.assert_array_equal(g, o.gain())
    np.testing.assert_array_equal(off, o.offset())
    np.testing.assert_array_equal(var, o.variance())


@pytest.mark.parametrize("shape", [1, 2])
def test_lane_shapes_match_oracle(lib_built, oracle_mod, shape):
    """Both voxel-group shapes for <= 64 views (16 lanes x 4 views, 32 lanes x 2 views)."""
    e, o, p, y = pair(lib_built, oracle_mod, lane_shape=shape)
    e.prepare()
    assert e.status().lane_shape == shape
    o.prepare()
    rows, stride = e.schedule(0)
    sg = e.sweep(0, 0)
    so = o.sweep_slices(rows, stride, 0, 0)
    assert sg[3] == so[3]
    assert rel(e.volume(), o.volume()) <= 1e-5


def test_autotuned_shape_is_valid_and_restores_state(lib_built, oracle_mod):
    """lane_shape = 0: trial passes on a snapshot choose the shape; the state after prepare is
    the untouched initial state (the first sweep still matches the oracle)."""
    e, o, p, y = pair(lib_built, oracle_mod, lane_shape=0)
    e.prepare()
    assert e.status().lane_shape in (1, 2)
    o.prepare()
    assert rel(e.error_sinogram(), o.error()) <= 1e-5
    rows, stride = e.schedule(0)
    e.sweep(0, 0)
    o.sweep_slices(rows, stride, 0, 0)
    assert rel(e.volume(), o.volume()) <= 1e-5
