"""HAADF reconstruction with a bright-field tilt series (the reference's --brightfield,
initializeBrightFieldData, HAADF_ReconstructionEngine_Extra.cpp:84-176): the parallel engines
against the oracle (which reproduces the reference's own run bit for bit,
tests/test_oracle_vs_ref.py) from the same state and in the same visit order.

  error sinogram after set-up (FP32)                       ||d|| / ||ref||      <= 1e-5
  one parallel sweep, same order (FP32; FP64, float32
    read-out)                                              ||d|| / ||ref||      <= 1e-5; 1e-7
  offsets after the offset-only estimation                 max relative         <= 1e-6
  MAP cost over sweeps with offset and variance updates    non-increasing
  gains                                                    unchanged
"""
import os
import sys

import numpy as np
import pytest

from conftest import haadf_params

HERE = os.path.dirname(os.path.abspath(__file__))
pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-300))


def case():
    g = dict(np.load(os.path.join(HERE, "golden", "haadf_bf_assist_small.npz")))
    return g["counts"], g["bf_counts"], g["tilts"], float(g["thickness"])


def pair(mbir, oracle_mod, **kw):
    y, bf, ang, th = case()
    p = haadf_params(mbir, th, **kw)
    e = mbir.Engine(p)
    e.set_sinogram(y, ang)
    e.set_bright_field(bf)
    o = oracle_mod.Oracle(oracle_mod.params_from_mbir(p), y, ang)
    o.set_bf_assist(bf.astype(np.float64))
    return e, o


@pytest.mark.parametrize("precision,tol", [(0, 1e-5), (1, 1e-9)])
def test_parallel_sweep_with_bright_field_matches_oracle(lib_built, oracle_mod, precision, tol):
    mbir = lib_built
    e, o = pair(mbir, oracle_mod, precision=precision)
    e.prepare()
    o.prepare()
    assert rel(e.error_sinogram(), o.error()) <= max(tol, 1e-6)
    for k in range(2):
        rows, stride = e.schedule(k)
        sg = e.sweep(0, k)
        so = o.sweep_slices(rows, stride, 0, k)
        assert sg[3] == so[3] and sg[2] == so[2], (k, sg, so)
        # the volume is read out in float32
        assert rel(e.volume(), o.volume()) <= max(tol, 1e-7), (k, rel(e.volume(), o.volume()))
        assert rel(e.error_sinogram(), o.error()) <= max(tol, 1e-6), k
    g0, _, _ = e.nuisance()
    e.joint_estimation()
    o.joint_estimation()
    g1, off, _ = e.nuisance()
    np.testing.assert_array_equal(g0, g1)
    np.testing.assert_allclose(off, o.offset(), rtol=1e-6)
    assert rel(e.error_sinogram(), o.error()) <= max(tol, 1e-6)
    e.close()


def test_cost_with_bright_field_non_increasing(lib_built, oracle_mod):
    mbir = lib_built
    e, o = pair(mbir, oracle_mod)
    e.prepare()
    costs = [e.cost()[0]]
    for k in range(6):
        e.sweep(k, 0)
        e.joint_estimation()
        e.update_weights()
        costs.append(e.cost()[0])
    e.close()
    assert all(b <= a * (1 + 1e-7) for a, b in zip(costs, costs[1:])), costs


def test_bright_field_size_mismatch_refused(lib_built):
    mbir = lib_built
    y, bf, ang, th = case()
    e = mbir.Engine(haadf_params(mbir, th))
    e.set_sinogram(y, ang)
    with pytest.raises(mbir.MbirError) as ei:
        e.set_bright_field(bf[:, :-1, :])
    assert "not matched" in str(ei.value)
    e.close()
