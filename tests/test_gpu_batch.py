"""Batched execution: many reconstructions of uneven size in one persistent launch per sweep
give the same result as each reconstruction run alone, within the FP32 tolerance."""
import numpy as np
import pytest

from conftest import haadf_params

pytestmark = pytest.mark.gpu


def series(mbir, seed, n_r, n_t, views, max_deg, thickness):
    import synthetic
    ang = synthetic.tilt_angles(max_deg, 2 * max_deg / (views - 1))
    rng = np.random.default_rng(seed)
    shapes = [(rng.uniform(-n_r / 4, n_r / 4), rng.uniform(-n_t / 4, n_t / 4),
               rng.uniform(-thickness / 3, thickness / 3), a, a, a, rng.uniform(0.5, 2))
              for a in rng.uniform(3, 8, 4)]
    proj = synthetic.ellipsoid_projection(ang, n_r, n_t, shapes)
    y, _ = synthetic.haadf_measurements(proj, seed=seed)
    return y, ang.astype(np.float32), thickness


CASES = [(1, 96, 12, 41, 70.0, 16.0), (2, 64, 20, 51, 60.0, 12.0), (3, 128, 8, 61, 65.0, 20.0),
         (4, 80, 16, 45, 60.0, 10.0)]


def make_engines(mbir):
    out = []
    for (seed, n_r, n_t, views, mx, th) in CASES:
        y, ang, th = series(mbir, seed, n_r, n_t, views, mx, th)
        e = mbir.Engine(haadf_params(mbir, th))
        e.set_sinogram(y, ang)
        e.prepare()
        out.append(e)
    return out


def rel(a, b):
    return float(np.linalg.norm(a.astype(np.float64) - b) / max(np.linalg.norm(b), 1e-300))


def test_batched_sweeps_match_single(lib_built):
    mbir = lib_built
    alone = make_engines(mbir)
    batched = make_engines(mbir)
    with mbir.Batch(0) as b:
        for e in batched:
            b.add(e)
        for k in range(3):
            st_b = b.sweep(outer=k)
            st_s = np.stack([e.sweep(k, 0) for e in alone])
            np.testing.assert_array_equal(st_b[:, 2:], st_s[:, 2:])  # skipped / updated counts
        assert b.last_ms() > 0
    for ea, eb in zip(alone, batched):
        assert rel(eb.volume(), ea.volume()) <= 1e-5
        assert rel(eb.error_sinogram(), ea.error_sinogram()) <= 1e-5


def test_batch_slice_group_tuning(lib_built):
    """The batch tunes its CTA size online over its second to fifth sweeps (512, 256, 256, 512
    threads) and keeps one; the results are those of a fixed CTA size, bit for bit."""
    mbir = lib_built
    tuned, fixed = make_engines(mbir), make_engines(mbir)
    with mbir.Batch(0) as bt, mbir.Batch(0) as bx:
        for e in tuned:
            bt.add(e)
        for e in fixed:
            bx.add(e)
        bx.set_threads(512)
        seen = []
        for k in range(7):
            seen.append(bt.threads())
            np.testing.assert_array_equal(bt.sweep(outer=k), bx.sweep(outer=k))
        assert seen[:5] == [0] * 5 and seen[5] in (256, 512) and seen[6] == seen[5], seen
    for a, b in zip(tuned, fixed):
        np.testing.assert_array_equal(a.volume(), b.volume())
        np.testing.assert_array_equal(a.error_sinogram(), b.error_sinogram())


def test_batch_run_to_tolerance(lib_built):
    mbir = lib_built
    engines = make_engines(mbir)
    with mbir.Batch(0) as b:
        for e in engines:
            b.add(e)
        outer, cost = b.run(40, 1e-4)
    assert np.all(outer >= 2) and np.all(np.isfinite(cost))
    for e, c in zip(engines, cost):
        tot, _ = e.cost()
        assert abs(tot - c) <= 1e-9 * abs(c)


def test_batch_rejects_fp64_and_reference_order(lib_built):
    mbir = lib_built
    y, ang, th = series(mbir, 9, 64, 8, 41, 60.0, 12.0)
    for kw in ({"precision": mbir.FP64}, {"order_mode": mbir.ORDER_REFERENCE}):
        e = mbir.Engine(haadf_params(mbir, th, **kw))
        e.set_sinogram(y, ang)
        e.prepare()
        with mbir.Batch(0) as b:
            with pytest.raises(mbir.MbirError):
                b.add(e)
        e.close()


def make_mixed(mbir):
    """Two HAADF and two bright-field reconstructions of different sizes."""
    from conftest import bf_case, bf_params
    out = make_engines(mbir)[:2]
    for (n_r, n_t, seed) in ((64, 8, 5), (48, 12, 6)):
        y, ang, th = bf_case(n_r=n_r, n_t=n_t, seed=seed)
        e = mbir.Engine(bf_params(mbir, th))
        e.set_sinogram(y, ang)
        e.prepare()
        out.append(e)
    return out


def test_batched_mixed_haadf_bf_match_single(lib_built):
    """HAADF sweeps and bright-field NHICD calls in one persistent launch give the same bits as
    each engine alone (same lists, same order, same arithmetic)."""
    mbir = lib_built
    alone = make_mixed(mbir)
    batched = make_mixed(mbir)
    with mbir.Batch(0) as b:
        for e in batched:
            b.add(e)
        for k in range(4):
            st_b = b.sweep(outer=k)
            st_s = np.stack([e.sweep(k, 0) for e in alone])
            np.testing.assert_array_equal(st_b[:, 2:], st_s[:, 2:])
    for ea, eb in zip(alone, batched):
        assert np.array_equal(eb.volume(), ea.volume())
        assert np.array_equal(eb.error_sinogram(), ea.error_sinogram())
    for ea, eb in zip(alone[2:], batched[2:]):
        np.testing.assert_array_equal(eb.call_lines(), ea.call_lines())
        np.testing.assert_array_equal(eb.bf_state()[0], ea.bf_state()[0])  # selectors


def test_batched_bf_uneven_views_match_single(lib_built):
    """Bright-field engines with different view counts in one batch: their per-call colour
    schedules are built side by side on host threads with different shared-memory sizes (the
    kernels' size limit is set once, to the device maximum, so concurrent set-ups cannot race),
    and every engine gives the same bits as alone."""
    mbir = lib_built
    from conftest import bf_case, bf_params

    def make():
        out = []
        for (n_r, n_t, seed, step) in ((64, 8, 5, 4.0), (48, 10, 6, 3.0), (56, 6, 7, 2.0),
                                       (40, 12, 8, 6.0)):
            y, ang, th = bf_case(n_r=n_r, n_t=n_t, seed=seed, step=step)
            e = mbir.Engine(bf_params(mbir, th))
            e.set_sinogram(y, ang)
            e.prepare()
            out.append(e)
        return out

    alone, batched = make(), make()
    assert len({e.dims()[3] for e in alone}) == 4  # four view counts
    with mbir.Batch(0) as b:
        for e in batched:
            b.add(e)
        for k in range(6):
            st_b = b.sweep(outer=k)
            st_s = np.stack([e.sweep(k, 0) for e in alone])
            np.testing.assert_array_equal(st_b[:, 2:], st_s[:, 2:])
    for ea, eb in zip(alone, batched):
        assert np.array_equal(eb.volume(), ea.volume())
        np.testing.assert_array_equal(eb.call_lines(), ea.call_lines())
