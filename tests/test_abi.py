"""The C-ABI library: loads, exports every declared symbol, parameter layout, host-side setup.

These run without a GPU: nothing here launches a kernel."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from conftest import ROOT, haadf_params, small_case


def declared_functions():
    src = open(os.path.join(ROOT, "include", "mbir_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(mbir_[a-z_0-9]+)\s*\(", src)))


def test_library_exports_every_declared_symbol(lib_built):
    mbir = lib_built
    names = declared_functions()
    assert len(names) >= 25
    L = mbir.lib()
    for n in names:
        assert hasattr(L, n), f"{n} declared in include/mbir_gb300.h but not exported"
    assert set(names) == set(mbir.SIGNATURES), "binding and header disagree"


def test_params_layout_and_defaults(lib_built):
    mbir = lib_built
    p = mbir.default_params()
    assert p.struct_size == C.sizeof(mbir.MbirParams)
    # InitializeAdvancedParams (HAADF_ReconstructionEngine.cpp:244-259)
    assert p.x_shrink_factor == 0.6 and p.z_stretch == 2
    assert p.detector_response_bins == 64 and p.profile_resolution == 1536
    assert p.beam_resolution == 512 and p.joint_estimation == 1 and p.zero_skipping == 1
    assert p.noise_model == 1 and p.estimate_prior == 0 and p.noise_estimation == 0
    # HAADF_QGGMRFPriorModel.cpp:12-15
    assert p.qggmrf_p == 2.0 and p.qggmrf_c == 0.001 and p.qggmrf_alpha == 1.5
    # CLI defaults (HAADFReconstructionArgsParser.cpp:155-185)
    assert abs(p.diffuseness - 0.2) < 1e-12 and p.num_resolutions == 3
    assert p.outer_iterations == 30 and p.inner_iterations == 10
    assert abs(p.stop_threshold - 0.005) < 1e-12 and p.default_variance == 1.0
    bf = mbir.default_params(mbir.BF)
    assert bf.qggmrf_c == 0.01


def test_create_rejects_bad_params(lib_built):
    mbir = lib_built
    p = mbir.default_params()
    p.struct_size = 12
    with pytest.raises(mbir.MbirError):
        mbir.Engine(p)
    p = mbir.default_params()
    p.sigma_x = 0.0
    with pytest.raises(mbir.MbirError):
        mbir.Engine(p)


def test_set_sinogram_validation_and_dims(lib_built, oracle_mod):
    mbir = lib_built
    y, ang, th = small_case()
    p = haadf_params(mbir, th)
    with mbir.Engine(p) as e:
        with pytest.raises(mbir.MbirError):
            e.set_sinogram(y[:, :, :0], ang)
        e.set_sinogram(y, ang)
        nz, nx, ny, nt, nr, ntt = e.dims()
        assert (nt, nr, ntt) == y.shape
        o = oracle_mod.Oracle(oracle_mod.params_from_mbir(p), y, ang)
        assert (nz, nx, ny) == (o.nz, o.nx, o.ny)
        with pytest.raises(mbir.MbirError) as ei:
            e.sweep()
        assert ei.value.code == -5  # ESTATE: prepare first


@pytest.mark.parametrize("levels,level", [(1, -1), (2, 0), (3, 0), (3, 1)])
def test_geometry_levels_match_oracle(lib_built, oracle_mod, levels, level):
    mbir = lib_built
    y, ang, th = small_case(n_r=64, n_t=12)
    p = haadf_params(mbir, th, num_resolutions=levels, level=level)
    with mbir.Engine(p) as e:
        e.set_sinogram(y, ang)
        o = oracle_mod.Oracle(oracle_mod.params_from_mbir(p), y, ang)
        assert e.dims()[:3] == (o.nz, o.nx, o.ny)


def test_host_tables_match_oracle(lib_built, oracle_mod):
    """Detector response H and H_t are FP64 on both sides and built by the same formulas."""
    mbir = lib_built
    y, ang, th = small_case()
    p = haadf_params(mbir, th)
    with mbir.Engine(p) as e:
        e.set_sinogram(y, ang)
        H, Ht = e.tables()
        o = oracle_mod.Oracle(oracle_mod.params_from_mbir(p), y, ang)
        np.testing.assert_allclose(H, o.detector_response(), rtol=1e-12, atol=1e-15)
        np.testing.assert_allclose(Ht, o.ht(), rtol=1e-12, atol=1e-15)
        g, off, var = e.nuisance()
        o.init_nuisance()
        np.testing.assert_allclose(g, o.gain(), rtol=1e-12)
        np.testing.assert_allclose(off, o.offset(), rtol=1e-10)


def test_schedule_is_conflict_free(lib_built, oracle_mod):
    """Voxels x and x+stride of any row never share a detector bin at any view (checked
    against the oracle's FP64 A-matrix columns), and the row order is a permutation."""
    mbir = lib_built
    y, ang, th = small_case()
    p = haadf_params(mbir, th)
    with mbir.Engine(p) as e:
        e.set_sinogram(y, ang)
        rows, stride = e.schedule(0)
        nz, nx = e.dims()[:2]
        assert sorted(rows.tolist()) == list(range(nz))
        assert 2 <= stride < nx
        o = oracle_mod.Oracle(oracle_mod.params_from_mbir(p), y, ang)
        for z in range(0, nz, 3):
            cols = [set(o.amatrix_column(z, x)[0].tolist()) for x in range(nx)]
            for x in range(nx - stride):
                for m in range(1, (nx - x - 1) // stride + 1):
                    assert not (cols[x] & cols[x + m * stride]), (z, x, m)


def test_mrc_load_matches_direct(lib_built, tmp_path):
    """MRC in (FEI extended header: tilts + pixel size) gives the same sinogram as set_sinogram."""
    mbir = lib_built
    import synthetic
    y, ang, th = small_case(n_r=32, n_t=6)
    path = tmp_path / "series.mrc"
    synthetic.write_tilt_series_mrc(str(path), y, ang, pixel_size_nm=1.0)
    p = haadf_params(mbir, th)
    with mbir.Engine(p) as e:
        e.load_mrc(path)
        assert e.dims()[3:] == y.shape
        H1, _ = e.tables()
    # the pixel size travels as float32 metres and is scaled by 1e9 in double
    # (MRCSinogramInitializer.cpp:207-211), so the pitch is float(1e-9)*1e9, not exactly 1
    dr = float(np.float32(1e-9)) * 1.0e9
    with mbir.Engine(p) as e2:
        e2.set_sinogram(y, ang, dr, dr)
        H2, _ = e2.tables()
    np.testing.assert_array_equal(H1, H2)


def test_mrc_subvolume_and_excluded_views(lib_built, tmp_path):
    mbir = lib_built
    import synthetic
    y, ang, th = small_case(n_r=40, n_t=9)
    path = tmp_path / "s.mrc"
    synthetic.write_tilt_series_mrc(str(path), y, ang, mode=2)
    p = haadf_params(mbir, th)
    p.use_subvolume = 1
    # x 4..35 is symmetric about the centre 20; y 0..5 has 6 rows (a multiple of 3)
    for i, v in enumerate([4, 0, 0, 35, 5, len(ang) - 1]):
        p.subvolume[i] = v
    p.n_excluded_views = 2
    p.excluded_views[0] = 1
    p.excluded_views[1] = 3
    with mbir.Engine(p) as e:
        e.load_mrc(path)
        assert e.dims()[3:] == (len(ang) - 2, 32, 6)


def test_mrc_errors(lib_built, tmp_path):
    mbir = lib_built
    p = haadf_params(mbir, 16.0)
    with mbir.Engine(p) as e:
        with pytest.raises(mbir.MbirError) as ei:
            e.load_mrc(tmp_path / "missing.mrc")
        assert ei.value.code == -4
        bad = tmp_path / "bad.mrc"
        bad.write_bytes(b"\0" * 100)
        with pytest.raises(mbir.MbirError):
            e.load_mrc(bad)


def test_server_reports_device_failure_without_gpu(lib_built):
    """Failure path of the serving loop, exercised on the host: with no usable device the
    request is admitted, its preparation fails, and it is retired with an error code instead of
    hanging the queue."""
    import conftest
    if conftest.has_gpu():
        pytest.skip("a GPU is present: the failure path needs a host without one")
    mbir = lib_built
    y, ang, th = small_case(n_r=32, n_t=4)
    with mbir.Server(0, 1 << 30, 0) as s:
        rid = s.submit(haadf_params(mbir, th), y, ang, max_outer=2, tol=0.0)
        with pytest.raises(mbir.MbirError):
            s.wait(rid, timeout=30.0)
        state = s.poll(rid)[0]
        assert state < 0
        assert s.stats().failed == 1


def test_server_rejects_oversized_request(lib_built):
    mbir = lib_built
    y, ang, th = small_case(n_r=32, n_t=4)
    with mbir.Server(0, 1024, 0) as s:
        with pytest.raises(mbir.MbirError) as ei:
            s.submit(haadf_params(mbir, th), y, ang)
        assert ei.value.code == -2
