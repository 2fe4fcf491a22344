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

    def slice_rows(self):
        out = []
        for y in range(self.o.ny):
            t0, val = self.o.voxel_line_response(y)
            out.append((t0, len(val)))
        return out


class LostRankBackend(OracleBackend):
    """A rank whose host fails after `fail_after` sweeps: it raises between sweeps, with none
    of its work in flight, and its process leaves the group."""

    def __init__(self, o, schedule, fail_after):
        super().__init__(o, schedule)
        self.fail_after = fail_after

    def sweep_colour(self, colour, outer, inner):
        if colour == 0 and self.sweeps == self.fail_after:
            raise RuntimeError("injected host failure")
        return super().sweep_colour(colour, outer, inner)


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


class OracleOwnedBackend(OracleBackend):
    """An oracle rank that holds only its slab's slices, one halo plane on each side and their
    detector rows (shard.owned_slab), with the drivers' global slice indices mapped to its own."""

    def __init__(self, o, schedule, dims, base):
        super().__init__(o, schedule)
        self.dims_g = tuple(dims)
        self.base = base

    def dims(self):
        return self.dims_g

    def set_slab(self, y0, y1):
        super().set_slab(y0 - self.base, y1 - self.base)

    def get_planes(self, y, n):
        return super().get_planes(y - self.base, n)

    def set_planes(self, y, planes):
        super().set_planes(y - self.base, planes)


def _owned_problem(world, rank):
    import mbir
    import oracle
    import shard
    from conftest import haadf_params, small_case
    y, ang, th = small_case(n_t=16)
    p = haadf_params(mbir, th)
    e = mbir.Engine(p)  # host-only use: geometry, schedule, the initial nuisance of the series
    e.set_sinogram(y, ang)
    dims = e.dims()
    nuis = e.nuisance()
    (y0, y1), base, top = shard.owned_slab(dims[2], world, rank)
    o = oracle.Oracle(oracle.params_from_mbir(p), np.ascontiguousarray(y[:, :, base:top]), ang)
    o.prepare()
    o.apply_nuisance(*nuis)
    return e, o, p, dims, base, nuis


def _rank_owned(rank, world, port, q):
    import sys
    here = os.path.dirname(os.path.abspath(__file__))
    root = os.path.dirname(here)
    for d in (os.path.join(root, "openmbir-tem_gb300"), os.path.join(root, "oracle"), here):
        sys.path.insert(0, d)
    import torch
    import torch.distributed as dist
    import shard
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=world)
    try:
        e, o, p, dims, base, _ = _owned_problem(world, rank)
        be = OracleOwnedBackend(o, e.schedule, dims, base)
        (y0, y1), hist = shard.run_sharded(dist, be, 3, p.target_gain)
        vol = np.zeros((dims[0], dims[1], dims[2]))
        vol[:, :, y0:y1] = o.volume()[:, :, y0 - base:y1 - base]
        t = torch.from_numpy(vol)
        dist.all_reduce(t)
        if rank == 0:
            q.put((t.numpy(), o.gain().copy(), o.offset().copy(), o.variance().copy(),
                   np.array(hist)))
    finally:
        dist.destroy_process_group()


def test_owned_slabs_two_cpu_ranks_match_single_process(oracle_mod, lib_built):
    """Ranks that hold only their slab, one halo plane each side and those slices' detector
    rows (16 slices over two ranks: 9 and 10 slices held) give one process's result."""
    vol, g, off, var, hist = _run_ranks(_rank_owned, 2)
    e, o, p, dims, base, nuis = _owned_problem(1, 0)
    assert base == 0 and o.ny == dims[2]
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


class OracleBFBackend(OracleBackend):
    """Bright-field oracle ranks: every call takes all lines (no NHICD lists) in the engine's
    row order; the slab's rows are its slices' rows (delta_xy = delta_t)."""

    def bf_call_begin(self, outer, inner):
        self.active = np.ones(self.o.nz * self.o.nx, np.uint8)
        self.rows, self.stride = self.schedule(self.sweeps)
        self.o.bf_reset_mag(self.active)

    def sweep_colour(self, colour, outer, inner):
        return self.o.bf_sweep_colour(self.active, self.rows, self.stride, colour, self.y0,
                                      self.y1, outer, inner)

    def bf_call_magnitudes(self):
        return np.where(self.active.reshape(self.o.nz, self.o.nx) != 0, self.o.mag_map(), 0.0)

    def bf_call_end(self, magnitudes):
        act = self.active.reshape(self.o.nz, self.o.nx) != 0
        self.o.mag_map()[act] = np.asarray(magnitudes).reshape(self.o.nz, self.o.nx)[act]
        self.sweeps += 1

    def roi_sums(self):
        return np.array([self.o.roi_mag_sum(), self.o.roi_volume_sum_range(self.y0, self.y1)])

    def bf_slab_sums(self, kind):
        if kind == 2:
            return self.o.bf_offset_sums(self.y0, self.y1)
        return self.o.bf_variance_sums(self.y0, self.y1)

    def bf_slab_apply(self, kind, sums):
        if kind == 2:
            self.o.bf_apply_offsets(sums, self.y0, self.y1)
        else:
            self.o.bf_apply_variance(sums, self.y0, self.y1)


def _rank_bf(rank, world, port, q):
    import sys
    here = os.path.dirname(os.path.abspath(__file__))
    root = os.path.dirname(here)
    for d in (os.path.join(root, "openmbir-tem_gb300"), os.path.join(root, "oracle"), here):
        sys.path.insert(0, d)
    import torch
    import torch.distributed as dist
    import mbir
    import oracle
    import shard
    from conftest import bf_case, bf_params
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=world)
    try:
        y, ang, th = bf_case(n_r=48, n_t=6)
        p = bf_params(mbir, th, nhicd=0)
        e = mbir.Engine(p)  # host-only use: geometry and schedule
        e.set_sinogram(y, ang)
        o = oracle.Oracle(oracle.params_from_mbir(p), y, ang)
        o.prepare()
        be = OracleBFBackend(o, e.schedule)
        (y0, y1), hist = shard.run_sharded_bf(dist, be, 3, nhicd=False)
        vol = np.zeros((o.nz, o.nx, o.ny))
        vol[:, :, y0:y1] = o.volume()[:, :, y0:y1]
        t = torch.from_numpy(vol)
        dist.all_reduce(t)
        if rank == 0:
            q.put((t.numpy(), o.offset().copy(), o.variance().copy(), o.mag_map().copy(),
                   np.array(hist)))
    finally:
        dist.destroy_process_group()


class OracleOwnedBFBackend(OracleBFBackend):
    """A bright-field oracle rank holding only its slab, halo planes and their detector rows."""

    def __init__(self, o, schedule, dims, base):
        super().__init__(o, schedule)
        self.dims_g = tuple(dims)
        self.base = base

    def dims(self):
        return self.dims_g

    def set_slab(self, y0, y1):
        super().set_slab(y0 - self.base, y1 - self.base)

    def get_planes(self, y, n):
        return super().get_planes(y - self.base, n)

    def set_planes(self, y, planes):
        super().set_planes(y - self.base, planes)


def _rank_owned_bf(rank, world, port, q):
    import sys
    here = os.path.dirname(os.path.abspath(__file__))
    root = os.path.dirname(here)
    for d in (os.path.join(root, "openmbir-tem_gb300"), os.path.join(root, "oracle"), here):
        sys.path.insert(0, d)
    import torch
    import torch.distributed as dist
    import mbir
    import oracle
    import shard
    from conftest import bf_case, bf_params
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=world)
    try:
        y, ang, th = bf_case(n_r=48, n_t=12)
        p = bf_params(mbir, th, nhicd=0)
        e = mbir.Engine(p)  # host-only use: geometry and schedule
        e.set_sinogram(y, ang)
        dims = e.dims()
        (y0, y1), base, top = shard.owned_slab(dims[2], world, rank)
        o = oracle.Oracle(oracle.params_from_mbir(p), np.ascontiguousarray(y[:, :, base:top]),
                          ang)
        o.prepare()
        be = OracleOwnedBFBackend(o, e.schedule, dims, base)
        (y0, y1), hist = shard.run_sharded_bf(dist, be, 3, nhicd=False)
        vol = np.zeros(dims[:3])
        vol[:, :, y0:y1] = o.volume()[:, :, y0 - base:y1 - base]
        t = torch.from_numpy(vol)
        dist.all_reduce(t)
        if rank == 0:
            q.put((t.numpy(), o.offset().copy(), o.variance().copy(), np.array(hist)))
    finally:
        dist.destroy_process_group()


def _run_ranks(target, world):
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=target, args=(r, world, port, q)) for r in range(world)]
    for pr in procs:
        pr.start()
    out = q.get(timeout=300)
    for pr in procs:
        pr.join(timeout=60)
        assert pr.exitcode == 0
    return out


def test_owned_slabs_bright_field_two_cpu_ranks_match_one_rank(oracle_mod, lib_built):
    """Bright-field ranks holding only their slab, halo planes and rows (12 slices over two
    ranks: 7 and 8 held) give the result of one rank holding the whole series; the variance
    sums carry the number of entries they cover, so the sub-problems' own row counts do not
    enter the variance."""
    vol2, off2, var2, hist2 = _run_ranks(_rank_owned_bf, 2)
    vol1, off1, var1, hist1 = _run_ranks(_rank_owned_bf, 1)
    np.testing.assert_array_equal(hist2[0][2:], hist1[0][2:])
    assert np.linalg.norm(vol2 - vol1) / np.linalg.norm(vol1) <= 1e-9
    np.testing.assert_allclose(off2, off1, rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(var2, var1, rtol=1e-9)


def test_two_cpu_ranks_bright_field_match_one_rank(oracle_mod, lib_built):
    """Bright-field slabs on two CPU ranks (FP64 oracle): per call both colours with halo
    exchange, the call's magnitude map added over ranks, offset and variance updates from sums
    over ranks; the same as one rank holding the whole volume (1e-9: only the order of the
    cross-rank sums differs)."""
    vol2, off2, var2, mag2, hist2 = _run_ranks(_rank_bf, 2)
    vol1, off1, var1, mag1, hist1 = _run_ranks(_rank_bf, 1)
    np.testing.assert_array_equal(hist2[0][2:], hist1[0][2:])  # same updates in the first call
    assert np.linalg.norm(vol2 - vol1) / np.linalg.norm(vol1) <= 1e-9
    np.testing.assert_allclose(off2, off1, rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(var2, var1, rtol=1e-9)
    np.testing.assert_allclose(mag2, mag1, rtol=1e-9, atol=1e-15)


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


def test_check_slab_rows_finds_shared_rows():
    import shard
    own = [(y, 1) for y in range(8)]
    shard.check_slab_rows(own, shard.slabs(8, 2))
    wide = [(y, 2) for y in range(8)]  # slice y covers rows y and y+1
    with pytest.raises(ValueError, match="share detector rows"):
        shard.check_slab_rows(wide, shard.slabs(8, 2))


def _rank_shared_rows(rank, world, port, q):
    import sys
    from datetime import timedelta
    here = os.path.dirname(os.path.abspath(__file__))
    root = os.path.dirname(here)
    for d in (os.path.join(root, "openmbir-tem_gb300"), os.path.join(root, "oracle"), here):
        sys.path.insert(0, d)
    import torch.distributed as dist
    import oracle
    import shard
    from conftest import small_case
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=world, timeout=timedelta(seconds=30))
    try:
        import mbir
        from conftest import haadf_params
        y, ang, th = small_case()
        p = haadf_params(mbir, th)
        # rectangular pixels: delta_r = 1.5 delta_t, so a voxel slice (delta_xy = delta_r)
        # spans one and a half detector rows and neighbouring slices share a row
        o = oracle.Oracle(oracle.params_from_mbir(p), y, ang, 1.5, 1.0)
        be = OracleBackend(o, None)
        try:
            shard.run_sharded(dist, be, 1, p.target_gain)
            q.put((rank, "ran"))
        except ValueError as ex:
            q.put((rank, str(ex)))
    finally:
        dist.destroy_process_group()


def test_two_cpu_ranks_refuse_shared_boundary_rows(oracle_mod, lib_built):
    """Slabs whose edge slices share a detector row cannot own it: both ranks refuse before any
    exchange (the engine's set_slab answers MBIR_ENOTSUP for the same case)."""
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_shared_rows, args=(r, 2, port, q)) for r in range(2)]
    for pr in procs:
        pr.start()
    got = dict(q.get(timeout=300) for _ in range(2))
    for pr in procs:
        pr.join(timeout=60)
        assert pr.exitcode == 0
    assert all("share detector rows" in m for m in got.values()), got


def _rank_lost(rank, world, port, q):
    import sys
    import time
    from datetime import timedelta
    here = os.path.dirname(os.path.abspath(__file__))
    root = os.path.dirname(here)
    for d in (os.path.join(root, "openmbir-tem_gb300"), os.path.join(root, "oracle"), here):
        sys.path.insert(0, d)
    import torch.distributed as dist
    import shard
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=world, timeout=timedelta(seconds=10))
    e, o, p = _problem()
    be = LostRankBackend(o, e.schedule, 1) if rank == 1 else OracleBackend(o, e.schedule)
    t0 = time.time()
    try:
        shard.run_sharded(dist, be, 3, p.target_gain)
        q.put((rank, "finished", time.time() - t0))
    except Exception as ex:  # the survivor sees the lost peer as a failed collective
        q.put((rank, type(ex).__name__ + ": " + str(ex)[:200], time.time() - t0))
    q.close()
    q.join_thread()  # the message is on its way before the process leaves
    # no destroy_process_group: the failed rank leaves, as a crashed host would
    os._exit(0)


def test_lost_cpu_rank_fails_the_next_exchange(oracle_mod, lib_built):
    """Failure detection on CPU ranks: rank 1 fails between sweeps (after its first sweep, with
    nothing in flight) and leaves.  Rank 0 does not hang: its next exchange ends with an error
    within the process group's timeout."""
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_lost, args=(r, 2, port, q)) for r in range(2)]
    for pr in procs:
        pr.start()
    got = {}
    for _ in range(2):
        r, msg, dt = q.get(timeout=300)
        got[r] = (msg, dt)
    for pr in procs:
        pr.join(timeout=60)
    assert "injected host failure" in got[1][0]
    assert got[0][0] != "finished", got
    assert got[0][1] < 120, got
