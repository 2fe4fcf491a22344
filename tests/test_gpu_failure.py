"""Failure detection without a GPU fault: a bounded device wait that runs out reports
MBIR_ETIMEOUT and leaves the engines usable; a cancel from another thread ends a running
reconstruction with the reference's -999 between sweeps (HAADF_ReconstructionEngine.cpp:
401-416, 748, 834).  No test faults, traps or hangs the GPU: the wait that runs out is a
time-bounded spin on a counter that the test keeps below its target (the batch's colour-1 slices
wait for one colour-0 slice more than their series has), and its limit is half a second."""
import threading
import time

import numpy as np
import pytest

from conftest import haadf_params, small_case

pytestmark = pytest.mark.gpu

MBIR_ETIMEOUT = -6


def engine(mbir, **kw):
    y, ang, th = small_case()
    e = mbir.Engine(haadf_params(mbir, th, **kw))
    e.set_sinogram(y, ang)
    e.prepare()
    return e


def test_batch_wait_runs_out_and_engines_stay_usable(lib_built, monkeypatch):
    mbir = lib_built
    engines = [engine(mbir), engine(mbir)]
    with mbir.Batch(0) as b:
        for e in engines:
            b.add(e)
        b.set_wait_limit(0.5)
        monkeypatch.setenv("MBIR_TEST_UNMET_BATCH_WAIT", "1")
        t0 = time.perf_counter()
        with pytest.raises(mbir.MbirError) as ei:
            b.sweep(0)
        assert ei.value.code == MBIR_ETIMEOUT
        assert time.perf_counter() - t0 < 30
        monkeypatch.delenv("MBIR_TEST_UNMET_BATCH_WAIT")
        st = b.sweep(1)  # the next sweep runs normally
        assert np.all(np.isfinite(st))
    for e in engines:
        v = e.volume()
        assert np.all(np.isfinite(v)) and v.max() > 0
        e.sweep(2, 0)  # and each engine alone as well
        e.close()


def test_cancel_from_another_thread_mid_run(lib_built):
    mbir = lib_built
    e = engine(mbir, outer_iterations=5000)
    out = {}

    def work():
        try:
            e.run()
            out["rc"] = 0
        except mbir.MbirError as ex:
            out["rc"] = ex.code

    th = threading.Thread(target=work)
    th.start()
    t0 = time.perf_counter()
    while e.status().sweeps_done < 3 and time.perf_counter() - t0 < 60:
        time.sleep(0.01)
    e.cancel()
    th.join(timeout=120)
    assert not th.is_alive()
    assert out.get("rc") == -999, out
    done = e.status().sweeps_done
    assert 3 <= done < 5000
    assert np.all(np.isfinite(e.volume()))
    e.close()
