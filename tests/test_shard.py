"""y-slab sharding on CPU ranks (gloo, world size 2): the driver in openmbir-tem_gb300/shard.py
with the FP64 oracle as each rank's backend reproduces the single-process reconstruction (same
slices in the same colour order; only the summation order of the per-view sums differs)."""
import os
import socket

import numpy as np
import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


class OracleBackend:
    """Oracle ranks: the whole problem in FP64 on the host, only the slab swept and summed.
    The schedule (row order per sweep, x stride) is the engine's, computed on the host."""

    plane_dtype = np.float64

    def __init__(self, o, schedule):
        self.o = o
        self.schedule = schedule
        self.y0, self.y1 = 0, o.ny
        self.sweeps = 0
        self.rows = None

    def dims(self):
        return (self.o.nz, self.o.nx, self.o.ny) + tuple(self.o.shape)

    def set_slab(self, y0, y1):
        self.y0, self.y1 = y0, y1

    def sweep_colour(self, colour, outer, inner):
        if colour == 0:
            self.rows, self.stride = self.schedule(self.sweeps)
        st = self.o.sweep_colour(self.rows, self.stride, colour, self.y0, self.y1, outer, inner)
        if colour == 1:
            self.sweeps += 1
        return st

    def get_planes(self, y, n):
        return np.ascontiguousarray(self.o.volume()[:, :, y:y + n].transpose(2, 0, 1))

    def set_planes(self, y, planes):
        self.o.volume()[:, :, y:y + planes.shape[0]] = np.asarray(planes).transpose(1, 2, 0)

    def view_sums(self, kind):
        return self.o.view_sums(kind, self.y0, self.y1)  # t = y at delta_xy = delta_t

    def apply_nuisance(self, gain=None, offset=None, variance=None):
        if gain is not None:
            self.o.apply_nuisance(gain, offset, None)
        if variance is not None:
            self.o.apply_nuisance(self.o.gain().copy(), self.o.offset().copy(), variance)


def _problem():
    import mbir
    import oracle
    from conftest import haadf_params, small_case
    y, ang, th = small_case()
    p = haadf_params(mbir, th)
    e = mbir.Engine(p)  # host-only use: geometry and schedule
    e.set_sinogram(y, ang)
    o = oracle.Oracle(oracle.params_from_mbir(p), y, ang)
    o.prepare()
    return e, o, p


def _rank(rank, world, port, q):
    import sys
    here = os.path.dirname(os.path.abspath(__file__))
    root = os.path.dirname(here)
    for d in (os.path.join(root, "openmbir-tem_gb300"), os.path.join(root, "oracle"), here):
        sys.path.insert(0, d)
    import torch.distributed as dist
    import shard
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=world)
    try:
        e, o, p = _problem()
        be = OracleBackend(o, e.schedule)
        (y0, y1), hist = shard.run_sharded(dist, be, 3, p.target_gain)
        # get_planes hands out float32 planes; gather the FP64 slabs directly instead
        vol = np.zeros((o.nz, o.nx, o.ny))
        vol[:, :, y0:y1] = o.volume()[:, :, y0:y1]
        import torch
        t = torch.from_numpy(vol)
        dist.all_reduce(t)
        if rank == 0:
            q.put((t.numpy(), o.gain().copy(), o.offset().copy(), o.variance().copy(),
                   np.array(hist)))
    finally:
        dist.destroy_process_group()


def test_slabs_partition():
    import shard
    for n_y, world in ((8, 2), (9, 2), (7, 3), (2, 4)):
        s = shard.slabs(n_y, world)
        assert s[0][0] == 0 and s[-1][1] == n_y
        assert all(a[1] == b[0] for a, b in zip(s, s[1:]))
        sizes = [b - a for a, b in s]
        assert max(sizes) - min(sizes) <= 1


def test_two_cpu_ranks_match_single_process(oracle_mod, lib_built):
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for pr in procs:
        pr.start()
    vol, g, off, var, hist = q.get(timeout=300)
    for pr in procs:
        pr.join(timeout=60)
        assert pr.exitcode == 0
    # single process: the same sweeps (both colours), then gain/offset and variance updates
    e, o, p = _problem()
    for k in range(3):
        rows, stride = e.schedule(k)
        st = o.sweep_slices(rows, stride, k, 0)
        np.testing.assert_allclose(hist[k][2:], st[2:])
        o.joint_estimation()
        o.update_weights()
    ref = o.volume()
    assert np.linalg.norm(vol - ref) / np.linalg.norm(ref) <= 1e-9
    np.testing.assert_allclose(g, o.gain(), rtol=1e-9)
    np.testing.assert_allclose(off, o.offset(), rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(var, o.variance(), rtol=1e-9)
