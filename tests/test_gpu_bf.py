"""Bright-field parity: the sm_103a engine (C ABI) against the FP64 oracle's restatement of
BFForwardModel / BFUpdateYSlice / BFReconstructionEngine.

Tolerances (FP32 engine vs FP64 oracle, same state and order):
  error sinogram / weights after set-up          relative          <= 1e-5
  one NHICD call (volume, error, magnitudes)     ||d|| / ||ref||   <= 1e-5
  Bragg selector after a call or an update       entries differing <= 1e-4 of all
  offset / variance estimates from equal state   relative          <= 1e-6
  cost terms from equal state                    relative          <= 1e-6 (data), 1e-5 (prior)
  reference-exact FP64 run (calls + JE + UW)     bitwise (float32 read-out)
"""
import numpy as np
import pytest

from conftest import bf_case, bf_params

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-300))


def pair(mbir, oracle_mod, **kw):
    y, ang, th = bf_case()
    p = bf_params(mbir, th, **kw)
    e = mbir.Engine(p)
    e.set_sinogram(y, ang)
    o = oracle_mod.Oracle(oracle_mod.params_from_mbir(p), y, ang)
    return e, o, p, y


def sync_oracle(e, o):
    """Copy the engine's state into the oracle (float32 values, as doubles)."""
    sel, w, mag, _, t = e.bf_state()
    o.volume()[...] = e.volume()
    o.error()[...] = e.error_sinogram()
    o.selector()[...] = sel
    o.weight()[...] = w
    o.mag_map()[...] = mag
    o.set_bragg(t)


def test_bf_setup_matches_oracle(lib_built, oracle_mod):
    e, o, p, y = pair(lib_built, oracle_mod)
    e.prepare()
    o.prepare()
    g, off, var = e.nuisance()
    np.testing.assert_allclose(off, o.offset(), rtol=1e-12)  # -log(dosage), host FP64
    np.testing.assert_allclose(var, o.variance(), rtol=1e-12)
    sel, w, mag, _, t = e.bf_state()
    assert t == 3.0 and sel.all() and not mag.any()
    assert rel(w, o.weight()) <= 1e-6
    assert rel(e.error_sinogram(), o.error()) <= 1e-5


@pytest.mark.parametrize("precision,bragg,tol", [(0, 5.0e10, 1e-5), (1, 3.0, 1e-9)])
def test_bf_call_matches_oracle_same_order(lib_built, oracle_mod, precision, bragg, tol):
    """First two NHICD calls (homogeneous, then non-homogeneous) against the oracle's slice-order
    call over the same lines.  The Bragg selector is a threshold on |e sqrt(w)|: in the first
    calls almost every touched entry crosses T, so FP32 rounding flips decisions at the
    threshold and the FP32 engine is compared with the selector off (T = 5e10); the FP64 engine
    is compared at T = 3 with the selector switching."""
    e, o, p, y = pair(lib_built, oracle_mod, precision=precision, bragg_threshold=bragg,
                      call_schedule=0)
    e.prepare()
    o.prepare()
    nz, nx = e.dims()[:2]
    for k in range(2):
        rows, stride = e.schedule(k)
        sg = e.sweep(0, k)
        lines = e.call_lines()  # FP32: the coloured visit order; FP64: ascending (row walk)
        if k == 1:  # the NH list: lines whose filtered magnitude exceeds the 1/20 percentile
            o.bf_vsc()
            np.testing.assert_array_equal(np.sort(lines), o.bf_nh_lines(o.bf_nh_threshold()))
        active = np.zeros(nz * nx, np.uint8)
        active[lines] = 1
        if precision == 0:
            assert e.status().sched_levels > 0
            so = o.bf_sweep_slices_order(lines, 0, k)
        else:
            so = o.bf_sweep_slices(active, rows, stride, 0, k)
        assert sg[3] == so[3] and sg[2] == so[2], (k, sg, so)
        assert rel(e.volume(), o.volume()) <= max(tol, 1e-7), (k, rel(e.volume(), o.volume()))
        assert rel(e.error_sinogram(), o.error()) <= max(tol, 1e-7), k
        sel, w, mag, _, _ = e.bf_state()
        assert np.mean(sel != o.selector()) <= 1e-4
        assert rel(mag, o.mag_map()) <= max(tol, 1e-7), k


def test_bf_estimates_and_cost_match(lib_built, oracle_mod):
    e, o, p, y = pair(lib_built, oracle_mod)
    e.prepare()
    o.prepare()
    for k in range(3):
        e.sweep(0, k)
    sync_oracle(e, o)
    o.offset()[...] = e.nuisance()[1]
    o.variance()[...] = e.nuisance()[2]
    cg, pg = e.cost()
    co, po = o.bf_cost()
    np.testing.assert_allclose(pg[0], po[0], rtol=1e-6)
    np.testing.assert_allclose(pg[1], po[1], rtol=1e-5)
    np.testing.assert_allclose(pg[2], po[2], rtol=1e-12)
    e.joint_estimation()
    o.bf_joint_estimation()
    o.bf_update_selector()
    np.testing.assert_allclose(e.nuisance()[1], o.offset(), rtol=1e-6)
    assert rel(e.error_sinogram(), o.error()) <= 1e-5
    sync_oracle(e, o)
    e.update_weights()
    o.bf_update_weights()
    o.bf_update_selector()
    np.testing.assert_allclose(e.nuisance()[2], o.variance(), rtol=1e-6)
    sel, w, _, _, _ = e.bf_state()
    assert rel(w, o.weight()) <= 1e-6
    assert np.mean(sel != o.selector()) <= 1e-4


def test_bf_reference_exact_run_bitwise(lib_built, oracle_mod):
    """FP64 reference order: calls with the Bragg schedule (3 inner calls at T = 5e10, then T),
    offset and variance updates between outer iterations, NHICD lists; the volume rounds to the
    same float32 values as the oracle's."""
    mbir = lib_built
    e, o, p, y = pair(mbir, oracle_mod, order_mode=1, precision=mbir.FP64, outer_iterations=4,
                      inner_iterations=3, seed=31)
    e.run()
    o.prepare()
    n = o.bf_run(31, 0)
    assert n == e.status().sweeps_done == 6
    v = o.volume()
    assert np.array_equal(e.volume(), v.astype(np.float32)), rel(e.volume(), v)
    _, off, var = e.nuisance()
    np.testing.assert_array_equal(off, o.offset())
    np.testing.assert_array_equal(var, o.variance())


def test_bf_calls_decrease_cost(lib_built, oracle_mod):
    """With the nuisance parameters and T fixed, every ICD call lowers the BF MAP cost."""
    e, o, p, y = pair(lib_built, oracle_mod)
    e.prepare()
    costs = [e.cost()[0]]
    for k in range(8):
        e.sweep(0, k)
        costs.append(e.cost()[0])
    assert all(b <= a for a, b in zip(costs, costs[1:])), costs


@pytest.mark.parametrize("staging,shape", [(0, 1), (1, 1), (1, 2)])
def test_bf_level_schedule_bitwise_row_walk(lib_built, oracle_mod, staging, shape):
    """Level-scheduled NHICD calls give the row walk's bits: a run with the Bragg schedule,
    offset and variance updates and homogeneous and non-homogeneous lists, slices staged in
    shared memory or used in place in HBM; 16-lane and 32-lane voxel groups."""
    mbir = lib_built
    y, ang, th = bf_case()
    out = []
    for sched in (2, 1):
        p = bf_params(mbir, th, outer_iterations=3, inner_iterations=4, call_schedule=sched,
                      slice_staging=staging, seed=7, lane_shape=shape)
        e = mbir.Engine(p)
        e.set_sinogram(y, ang)
        e.run()
        st = e.status()
        sel, w, mag, _, _ = e.bf_state()
        out.append((e.volume(), e.error_sinogram(), sel, mag, e.nuisance(), st))
    (v0, e0, s0, m0, n0, st0), (v1, e1, s1, m1, n1, st1) = out
    assert st0.sched_levels > 0 and st1.sched_levels == 0
    assert st0.sweeps_done == st1.sweeps_done
    assert st0.voxels_updated == st1.voxels_updated
    assert st0.voxels_visited == st1.voxels_visited
    assert np.array_equal(v0, v1), rel(v0, v1)
    assert np.array_equal(e0, e1), rel(e0, e1)
    assert np.array_equal(s0, s1) and np.array_equal(m0, m1)
    for a, b in zip(n0, n1):
        np.testing.assert_array_equal(a, b)


def test_bf_device_colour_schedule_matches_host(lib_built, oracle_mod):
    """Each NHICD call's colour schedule, built on the device, equals the host definition
    (mbir_colour_schedule on the engine's footprint bins, the call's lines and the kernel's class
    cap of 32 voxel groups), its classes are independent, and the calls match the oracle run in
    that visit order (FP32, 1e-5; Bragg rejection off)."""
    mbir = lib_built
    e, o, p, y = pair(mbir, oracle_mod, call_schedule=0, bragg_threshold=5.0e10)
    e.prepare()
    o.prepare()
    lo, mask, ok = e.footprint_bins()
    nz, nx = ok.shape
    n_r = y.shape[1]
    for k in range(22):  # calls 20 and 22 reuse the cached schedules of sub-lists 0 and 1
        sg = e.sweep(0, k)
        lines, lofs = e.call_schedule()
        assert len(lines) > 0 and len(lofs) >= 2 and e.status().sched_levels == len(lofs) - 1
        act = np.zeros(nz * nx, np.uint8)
        act[lines] = 1
        hl, ho = mbir.colour_schedule(ok, lo, mask, 3, n_r, act.reshape(nz, nx), class_cap=32)
        np.testing.assert_array_equal(lines, hl)
        np.testing.assert_array_equal(lofs, ho)
        assert np.diff(lofs).max() <= 32
        np.testing.assert_array_equal(e.call_lines(), lines)
        if k >= 4:
            continue
        so = o.bf_sweep_slices_order(lines, 0, k)
        assert sg[3] == so[3] and sg[2] == so[2], (k, sg, so)
        assert rel(e.volume(), o.volume()) <= 1e-5, (k, rel(e.volume(), o.volume()))
        assert rel(e.error_sinogram(), o.error()) <= 1e-5, k


@pytest.mark.parametrize("n_r", [32, 48])
def test_bf_device_colour_schedule_short_calls(lib_built, n_r):
    """Calls of two and three 31-line blocks of the device colouring (~50 and ~75 lines: the
    first and last steps of its pipeline, a partial last block): the device schedule equals the
    host definition."""
    mbir = lib_built
    y, ang, th = bf_case(n_r=n_r, n_t=4)
    p = bf_params(mbir, th, call_schedule=0, bragg_threshold=5.0e10)
    e = mbir.Engine(p)
    e.set_sinogram(y, ang)
    e.prepare()
    lo, mask, ok = e.footprint_bins()
    nz, nx = ok.shape
    sizes = []
    for k in range(6):
        e.sweep(0, k)
        lines, lofs = e.call_schedule()
        sizes.append(len(lines))
        act = np.zeros(nz * nx, np.uint8)
        act[lines] = 1
        hl, ho = mbir.colour_schedule(ok, lo, mask, 3, y.shape[1], act.reshape(nz, nx),
                                      class_cap=32)
        np.testing.assert_array_equal(lines, hl)
        np.testing.assert_array_equal(lofs, ho)
    assert 31 < min(sizes) and max(sizes) < 3 * 31, sizes


@pytest.mark.parametrize("helpers,sequential", [("8", "0"), ("0", "0"), ("8", "1")])
def test_bf_device_colour_schedule_long_calls(lib_built, monkeypatch, helpers, sequential):
    """Calls of well over twenty 31-line blocks, so that the helper CTAs of the multi-CTA device
    colouring run ahead of the colouring CTA and each take several blocks: homogeneous and
    non-homogeneous calls give the host definition's schedule exactly, with helpers and without,
    and with the blocks' parallel greedy form and line by line."""
    mbir = lib_built
    monkeypatch.setenv("MBIR_COLOUR_HELPERS", helpers)
    monkeypatch.setenv("MBIR_COLOUR_SEQUENTIAL", sequential)
    y, ang, th = bf_case(n_r=512, n_t=4, thickness=64.0, n_particles=24)
    p = bf_params(mbir, th, call_schedule=0, bragg_threshold=5.0e10)
    with mbir.Engine(p) as e:
        e.set_sinogram(y, ang)
        e.prepare()
        lo, mask, ok = e.footprint_bins()
        nz, nx = ok.shape
        sizes = []
        for k in range(4):
            e.sweep(0, k)
            lines, lofs = e.call_schedule()
            sizes.append(len(lines))
            act = np.zeros(nz * nx, np.uint8)
            act[lines] = 1
            hl, ho = mbir.colour_schedule(ok, lo, mask, 3, y.shape[1], act.reshape(nz, nx),
                                          class_cap=32)
            np.testing.assert_array_equal(lines, hl)
            np.testing.assert_array_equal(lofs, ho)
    assert min(sizes) > 20 * 31, sizes
