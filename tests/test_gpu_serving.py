"""Served stream: requests admitted by device memory with continuous batching.  Each result must
be the same when the request is served alone and when it shares the device with others."""
import time

import numpy as np
import pytest

from conftest import haadf_params
from test_gpu_batch import CASES, series

pytestmark = pytest.mark.gpu


def requests(mbir):
    out = []
    for (seed, n_r, n_t, views, mx, th) in CASES:
        y, ang, th = series(mbir, seed, n_r, n_t, views, mx, th)
        out.append((haadf_params(mbir, th), y, ang))
    return out


def rel(a, b):
    return float(np.linalg.norm(a.astype(np.float64) - b) / max(np.linalg.norm(b), 1e-300))


def test_results_same_alone_and_in_the_mix(lib_built):
    mbir = lib_built
    reqs = requests(mbir)
    alone = []
    with mbir.Server(0, 0, 1) as s:  # one request on the device at a time
        for p, y, ang in reqs:
            rid = s.submit(p, y, ang, max_outer=12, tol=1e-4)
            s.wait(rid)
            alone.append((s.result(rid), s.poll(rid)[2]))
    with mbir.Server(0, 0, 0) as s:
        ids = []
        for p, y, ang in reqs:  # staggered arrivals: later requests join a running batch
            ids.append(s.submit(p, y, ang, max_outer=12, tol=1e-4))
            time.sleep(0.01)
        for rid in ids:
            s.wait(rid)
        mixed = [(s.result(rid), s.poll(rid)[2]) for rid in ids]
        st = s.stats()
        assert st.completed == len(reqs) and st.failed == 0
        assert 0 < st.p50_ms <= st.p99_ms
    for (va, na), (vm, nm) in zip(alone, mixed):
        assert na == nm
        assert rel(vm, va) <= 1e-5


def test_admission_respects_memory_budget(lib_built):
    """Each request's estimated footprint is measured alone; with a budget below their sum the
    server keeps some requests waiting, never exceeds the budget and admits in arrival order."""
    mbir = lib_built
    reqs = requests(mbir)
    sizes = []
    for p, y, ang in reqs:
        with mbir.Server(0, 0, 1) as s:
            s.wait(s.submit(p, y, ang, max_outer=1, tol=0.0))
            sizes.append(s.stats().peak_bytes)
    budget = max(sizes) + min(sizes) // 2
    assert budget < sum(sizes)
    with mbir.Server(0, budget, 0) as s:
        ids = [s.submit(p, y, ang, max_outer=3, tol=0.0) for p, y, ang in reqs]
        for rid in ids:
            s.wait(rid)
        lat = [s.poll(rid)[1] for rid in ids]
        assert all(l > 0 for l in lat)
        st = s.stats()
        assert st.budget_bytes == budget
        assert 0 < st.peak_bytes <= st.budget_bytes
        assert st.admitted == len(reqs) and st.admitted_out_of_order == 0
        assert st.peak_active < len(reqs)  # the budget kept some requests waiting


def test_mixed_haadf_bf_same_alone_and_in_the_mix(lib_built):
    """Bright-field and HAADF requests served together: each result equals the same request
    served alone (bright field converges per equivalent iteration of 20 calls)."""
    from conftest import bf_case, bf_params
    mbir = lib_built
    reqs = requests(mbir)[:2]
    for (n_r, n_t, seed) in ((64, 8, 5), (48, 12, 6)):
        y, ang, th = bf_case(n_r=n_r, n_t=n_t, seed=seed)
        reqs.append((bf_params(mbir, th), y, ang))
    outers = [6, 6, 40, 40]
    alone = []
    with mbir.Server(0, 0, 1) as s:
        for (p, y, ang), mo in zip(reqs, outers):
            rid = s.submit(p, y, ang, max_outer=mo, tol=1e-4)
            s.wait(rid)
            alone.append((s.result(rid), s.poll(rid)[2]))
    with mbir.Server(0, 0, 0) as s:
        ids = []
        for (p, y, ang), mo in zip(reqs, outers):
            ids.append(s.submit(p, y, ang, max_outer=mo, tol=1e-4))
            time.sleep(0.005)
        for rid in ids:
            s.wait(rid)
        mixed = [(s.result(rid), s.poll(rid)[2]) for rid in ids]
        assert s.stats().failed == 0
    for (va, na), (vm, nm) in zip(alone, mixed):
        assert na == nm
        assert np.array_equal(va, vm)
