"""mbir_set_observer: the engine's messages in the shape of the reference's
Observable::notify(msg, progress, aspect) (Code/MBIRLib/Common/Observable.h:65-101) --
"Calculating A Matrix....", "Starting Forward Projection", each intermediate image
(HAADF_ReconstructionEngine.cpp:757-763), "Reconstruction Complete" and every error, with the
reference's progress values and aspect numbers; and one JSON line of metrics per outer
iteration."""
import ctypes as C
import json
import os

import numpy as np
import pytest

from conftest import bf_case, bf_params, haadf_params, small_case

pytestmark = pytest.mark.gpu


def test_observer_messages_of_a_run_and_an_error(lib_built, tmp_path):
    mbir = lib_built
    y, ang, th = small_case()
    p = haadf_params(mbir, th, outer_iterations=3)
    seen = []
    with mbir.Engine(p) as e:
        e.set_sinogram(y, ang)
        e.set_intermediate_dir(str(tmp_path))
        e.set_observer(lambda m, prog, asp: seen.append((m, prog, asp)))
        e.run()
        assert seen[0] == ("Calculating A Matrix....", 0, mbir.UPDATE_PROGRESS_MESSAGE)
        assert seen[1] == ("Starting Forward Projection", 10,
                           mbir.UPDATE_PROGRESS_VALUE_AND_MESSAGE)
        images = [m for m, prog, asp in seen if asp == mbir.UPDATE_INTERMEDIATE_IMAGE]
        assert images == [os.path.join(str(tmp_path), f"{o}_0_ReconstructedVolume.rec")
                          for o in range(3)]
        assert all(os.path.exists(f) for f in images)
        assert seen[-1] == ("Reconstruction Complete", 100,
                            mbir.UPDATE_PROGRESS_VALUE_AND_MESSAGE)
        assert not any(asp == mbir.UPDATE_ERROR_MESSAGE for _, _, asp in seen)
        check_metrics(mbir, seen, 3, e.status())
        # an error reaches the observer with the text mbir_last_error gives
        n = len(seen)
        buf = np.zeros(1, np.float32)
        rc = mbir.lib().mbir_get_volume(e._h, buf.ctypes.data_as(C.POINTER(C.c_float)), 1)
        assert rc == -1
        assert seen[n:] == [(mbir.lib().mbir_last_error(e._h).decode(), 100,
                             mbir.UPDATE_ERROR_MESSAGE)]
        # removed: no more messages
        e.set_observer(None)
        rc = mbir.lib().mbir_get_volume(e._h, buf.ctypes.data_as(C.POINTER(C.c_float)), 1)
        assert rc == -1 and len(seen) == n + 1


def check_metrics(mbir, seen, n_outer, status):
    lines = [(json.loads(m), prog) for m, prog, asp in seen
             if asp == mbir.UPDATE_PROGRESS_MESSAGE and m.startswith("{")]
    assert [d["outer"] for d, _ in lines] == list(range(n_outer))
    assert [prog for _, prog in lines] == [100 * (k + 1) // n_outer for k in range(n_outer)]
    sweeps = [d["sweeps"] for d, _ in lines]
    assert sweeps == sorted(sweeps) and sweeps[-1] == status.sweeps_done
    upd = [d["voxels_updated"] for d, _ in lines]
    assert upd[0] > 0 and upd == sorted(upd) and upd[-1] == status.voxels_updated
    # rel_update divides by the ROI's sum |x| before the sweep: 0 for a sweep from a zero volume
    assert all(d["cost"] is None and d["rel_update"] >= 0 and d["icd_ms"] > 0 for d, _ in lines)


def test_observer_metrics_of_a_bright_field_run(lib_built):
    mbir = lib_built
    c, ang, th = bf_case()
    seen = []
    with mbir.Engine(bf_params(mbir, th, outer_iterations=3)) as e:
        e.set_sinogram(c, ang)
        e.set_observer(lambda m, prog, asp: seen.append((m, prog, asp)))
        e.run()
        assert seen[-1] == ("Reconstruction Complete", 100,
                            mbir.UPDATE_PROGRESS_VALUE_AND_MESSAGE)
        check_metrics(mbir, seen, 3, e.status())
