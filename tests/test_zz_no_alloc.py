"""mbir_error_view_sums_noalloc: per-view sums of squared errors on caller-owned device buffers
(no allocation; scratch in a static device array), checked through the C ABI against the
engine's own variance update (mbir_update_weights: alpha_v = sum_rt e^2 / (N_r N_t)).  Device
buffers here come from PyTorch (plumbing only).  Collected last, and runs alone as well."""
import ctypes as C

import numpy as np
import pytest

from conftest import haadf_params, small_case

pytestmark = pytest.mark.gpu


def noalloc_sums(mbir, err_host):
    import torch
    n_theta, n_r, n_t = err_host.shape
    ed = torch.from_numpy(np.ascontiguousarray(err_host, np.float32)).cuda()
    out = torch.full((n_theta,), float("nan"), dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    rc = mbir.lib().mbir_error_view_sums_noalloc(C.c_void_p(ed.data_ptr()), n_theta, n_r, n_t,
                                                 C.c_void_p(out.data_ptr()), C.c_void_p(stream))
    assert rc == 0
    torch.cuda.synchronize()
    return out.cpu().numpy()


def test_noalloc_view_sums_match_update_weights(lib_built):
    mbir = lib_built
    y, ang, th = small_case()
    with mbir.Engine(haadf_params(mbir, th)) as e:
        e.set_sinogram(y, ang)
        e.prepare()
        n_theta, n_r, n_t = e.dims()[3:]
        for k in range(2):  # two calls in a row, on different error sinograms
            e.sweep(0, k)
            err = e.error_sinogram()
            e.update_weights()
            alpha = e.nuisance()[2]
            sums = noalloc_sums(mbir, err)
            np.testing.assert_allclose(sums / (n_r * n_t), alpha, rtol=1e-6)


def test_noalloc_rejects_too_many_views(lib_built):
    mbir = lib_built
    import torch
    ed = torch.zeros(1025 * 4, dtype=torch.float32, device="cuda")
    out = torch.zeros(1025, dtype=torch.float64, device="cuda")
    rc = mbir.lib().mbir_error_view_sums_noalloc(C.c_void_p(ed.data_ptr()), 1025, 2, 2,
                                                 C.c_void_p(out.data_ptr()), None)
    assert rc == -1  # MBIR_EINVAL
