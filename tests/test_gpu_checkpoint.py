"""mbir_write_checkpoint / mbir_read_checkpoint: a HAADF run of N outer iterations and a run of
K < N, checkpointed to the reference's level hand-off files (ReconstructedObject.bin,
Final*Parameters.bin, FinalVariances.bin; HAADF_MultiResolutionReconstruction.cpp:212-222) plus
Checkpoint.bin and resumed to N by a new engine, give the same bits -- FP32 and FP64 parallel
order, and the reference order with a new visit order per sweep; checkpoints of another
configuration, missing files and bright field are refused."""
import numpy as np
import pytest

from conftest import bf_case, bf_params, haadf_params, small_case

pytestmark = pytest.mark.gpu


def straight_and_resumed(mbir, p, y, ang, tmp_path, n, k):
    p.outer_iterations = n
    with mbir.Engine(p) as e:
        e.set_sinogram(y, ang)
        e.run()
        vol, nui = e.volume64(), e.nuisance()
        sweeps = e.status().sweeps_done
    p.outer_iterations = k
    with mbir.Engine(p) as e:
        e.set_sinogram(y, ang)
        e.run()
        e.write_checkpoint(tmp_path)
    for name in ("ReconstructedObject.bin", "FinalGainParameters.bin",
                 "FinalOffsetParameters.bin", "FinalVariances.bin", "Checkpoint.bin"):
        assert (tmp_path / name).exists(), name
    p.outer_iterations = n
    with mbir.Engine(p) as e:
        e.set_sinogram(y, ang)
        e.read_checkpoint(tmp_path)
        e.run()
        vol2, nui2 = e.volume64(), e.nuisance()
        sweeps2 = e.status().sweeps_done
    return (vol, nui, sweeps), (vol2, nui2, sweeps2)


@pytest.mark.parametrize("mode", ["fp32_parallel", "fp64_parallel", "fp32_reference"])
def test_resumed_run_equals_straight_run(lib_built, tmp_path, mode):
    mbir = lib_built
    y, ang, th = small_case()
    if mode == "fp32_parallel":
        p = haadf_params(mbir, th)
    elif mode == "fp64_parallel":
        p = haadf_params(mbir, th, precision=mbir.FP64)
    else:
        p = haadf_params(mbir, th, order_mode=mbir.ORDER_REFERENCE,
                         seed_mode=mbir.SEED_PER_CALL)
    (vol, nui, sweeps), (vol2, nui2, sweeps2) = straight_and_resumed(mbir, p, y, ang, tmp_path,
                                                                     4, 2)
    assert sweeps == 4 and sweeps2 == 4
    np.testing.assert_array_equal(vol2, vol)
    for a, b in zip(nui2, nui):
        np.testing.assert_array_equal(a, b)


def test_checkpoint_refusals(lib_built, tmp_path):
    mbir = lib_built
    y, ang, th = small_case()
    p = haadf_params(mbir, th, outer_iterations=1)
    with mbir.Engine(p) as e:
        e.set_sinogram(y, ang)
        e.run()
        e.write_checkpoint(tmp_path)
    # another series size: a thicker sample has more z planes
    q = haadf_params(mbir, th * 2, outer_iterations=1)
    with mbir.Engine(q) as e:
        e.set_sinogram(y, ang)
        with pytest.raises(mbir.MbirError) as ex:
            e.read_checkpoint(tmp_path)
        assert ex.value.code == -1
        with pytest.raises(mbir.MbirError) as ex:
            e.read_checkpoint(tmp_path / "missing")
        assert ex.value.code == -4
    c, bang, bth = bf_case()
    with mbir.Engine(bf_params(mbir, bth)) as e:
        e.set_sinogram(c, bang)
        with pytest.raises(mbir.MbirError) as ex:
            e.read_checkpoint(tmp_path)
        assert ex.value.code == -7
