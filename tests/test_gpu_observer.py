"""mbir_set_observer: the engine's messages in the shape of the reference's
Observable::notify(msg, progress, aspect) (Code/MBIRLib/Common/Observable.h:65-101) --
"Calculating A Matrix....", "Starting Forward Projection", each intermediate image
(HAADF_ReconstructionEngine.cpp:757-763), "Reconstruction Complete" and every error, with the
reference's progress values and aspect numbers."""
import ctypes as C
import os

import numpy as np
import pytest

from conftest import haadf_params, small_case

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
