"""y-slab sharding through the C ABI: two ranks (spawned processes, gloo on host tensors), each
with its own engine on the GPU, sweep their slabs and exchange halo planes and per-view sums;
the result matches one engine running the whole volume.  The ranks only meet between kernel
launches (host-mediated), so they can share one GPU."""
import os
import socket

import numpy as np
import pytest

from conftest import bf_case, bf_params, haadf_params, small_case

pytestmark = pytest.mark.gpu


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, q):
    import sys
    here = os.path.dirname(os.path.abspath(__file__))
    root = os.path.dirname(here)
    for d in (os.path.join(root, "openmbir-tem_gb300"), os.path.join(root, "oracle"), here):
        sys.path.insert(0, d)
    import torch.distributed as dist
    import mbir
    import shard
    from conftest import bf_case, bf_params, haadf_params, small_case
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=world)
    try:
        y, ang, th = small_case()
        with mbir.Engine(haadf_params(mbir, th)) as e:
            e.set_sinogram(y, ang)
            e.prepare()
            be = shard.EngineBackend(e)
            (y0, y1), hist = shard.run_sharded(dist, be, 3, 1.0)
            vol = shard.gather_volume(dist, be, y0, y1)
            if rank == 0:
                q.put((vol, e.nuisance(), np.array(hist)))
    finally:
        dist.destroy_process_group()


def test_two_ranks_match_one_engine(lib_built):
    import multiprocessing as mp
    mbir = lib_built
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for pr in procs:
        pr.start()
    vol, (g, off, var), hist = q.get(timeout=300)
    for pr in procs:
        pr.join(timeout=120)
        assert pr.exitcode == 0
    y, ang, th = small_case()
    with mbir.Engine(haadf_params(mbir, th, outer_iterations=3)) as e:
        e.set_sinogram(y, ang)
        e.prepare()
        first = e.sweep(0, 0)
        np.testing.assert_array_equal(hist[0][2:], first[2:])  # same updates in sweep 1
    with mbir.Engine(haadf_params(mbir, th, outer_iterations=3)) as e:
        e.set_sinogram(y, ang)
        e.run()
        ref = e.volume()
        g1, off1, var1 = e.nuisance()
    r = float(np.linalg.norm(vol.astype(np.float64) - ref) / np.linalg.norm(ref))
    assert r <= 1e-4, r
    np.testing.assert_allclose(g, g1, rtol=1e-5)
    np.testing.assert_allclose(var, var1, rtol=1e-4)


BF_OUTER = 24  # more than one equivalent iteration of NHICD calls (20)


def _rank_bf(rank, world, port, q):
    import sys
    here = os.path.dirname(os.path.abspath(__file__))
    root = os.path.dirname(here)
    for d in (os.path.join(root, "openmbir-tem_gb300"), os.path.join(root, "oracle"), here):
        sys.path.insert(0, d)
    import torch.distributed as dist
    import mbir
    import shard
    from conftest import bf_case, bf_params
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=world)
    try:
        y, ang, th = bf_case()
        with mbir.Engine(bf_params(mbir, th, outer_iterations=BF_OUTER)) as e:
            e.set_sinogram(y, ang)
            e.prepare()
            be = shard.EngineBackend(e)
            (y0, y1), hist = shard.run_sharded_bf(dist, be, BF_OUTER)
            vol = shard.gather_volume(dist, be, y0, y1)
            if rank == 0:
                _, _, mag, _, _ = e.bf_state()
                q.put((vol, e.nuisance(), mag, np.array(hist)))
    finally:
        dist.destroy_process_group()


def test_two_ranks_bright_field_match_one_engine(lib_built):
    """Bright-field NHICD calls on two slabs (homogeneous and non-homogeneous lists, device
    colour schedules, offset and variance updates): the first call updates the same voxels as
    one engine, and the run ends where one engine's run ends (the cross-slab sums differ only in
    their order)."""
    import multiprocessing as mp
    mbir = lib_built
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_bf, args=(r, 2, port, q)) for r in range(2)]
    for pr in procs:
        pr.start()
    vol, (g, off, var), mag, hist = q.get(timeout=300)
    for pr in procs:
        pr.join(timeout=120)
        assert pr.exitcode == 0
    y, ang, th = bf_case()
    with mbir.Engine(bf_params(mbir, th, outer_iterations=BF_OUTER)) as e:
        e.set_sinogram(y, ang)
        e.prepare()
        first = e.sweep(0, 0)
        np.testing.assert_array_equal(hist[0][2:], first[2:])
    with mbir.Engine(bf_params(mbir, th, outer_iterations=BF_OUTER)) as e:
        e.set_sinogram(y, ang)
        e.run()
        ref = e.volume()
        _, off1, var1 = e.nuisance()
        _, _, mag1, _, _ = e.bf_state()
    r = float(np.linalg.norm(vol.astype(np.float64) - ref) / np.linalg.norm(ref))
    assert r <= 1e-4, r
    np.testing.assert_allclose(off, off1, rtol=1e-5)
    np.testing.assert_allclose(var, var1, rtol=1e-4)
    assert float(np.linalg.norm(mag - mag1) / np.linalg.norm(mag1)) <= 1e-3


def _rank_owned(rank, world, port, q):
    import sys
    here = os.path.dirname(os.path.abspath(__file__))
    root = os.path.dirname(here)
    for d in (os.path.join(root, "openmbir-tem_gb300"), os.path.join(root, "oracle"), here):
        sys.path.insert(0, d)
    import torch.distributed as dist
    import mbir
    import shard
    from conftest import haadf_params, small_case
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=world)
    try:
        y, ang, th = small_case(n_t=16)
        be = shard.OwnedSlabBackend.make(mbir, haadf_params(mbir, th), y, ang, world, rank)
        try:
            held = be.e.dims()[2]
            (y0, y1), hist = shard.run_sharded(dist, be, 3, 1.0)
            vol = shard.gather_volume(dist, be, y0, y1)
            if rank == 0:
                q.put((vol, be.e.nuisance(), np.array(hist), held))
        finally:
            be.close()
    finally:
        dist.destroy_process_group()


def test_two_owned_slab_ranks_match_one_engine(lib_built):
    """Each rank's engine holds only its slab, one halo plane on each side and their detector
    rows (16 slices over two ranks: rank 0 holds 9); the result matches one engine holding the
    whole series."""
    import multiprocessing as mp
    mbir = lib_built
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_owned, args=(r, 2, port, q)) for r in range(2)]
    for pr in procs:
        pr.start()
    vol, (g, off, var), hist, held = q.get(timeout=300)
    for pr in procs:
        pr.join(timeout=120)
        assert pr.exitcode == 0
    y, ang, th = small_case(n_t=16)
    assert held == 9
    with mbir.Engine(haadf_params(mbir, th, outer_iterations=3)) as e:
        e.set_sinogram(y, ang)
        e.prepare()
        first = e.sweep(0, 0)
        np.testing.assert_array_equal(hist[0][2:], first[2:])
    with mbir.Engine(haadf_params(mbir, th, outer_iterations=3)) as e:
        e.set_sinogram(y, ang)
        e.run()
        ref = e.volume()
        g1, off1, var1 = e.nuisance()
    r = float(np.linalg.norm(vol.astype(np.float64) - ref) / np.linalg.norm(ref))
    assert r <= 1e-4, r
    np.testing.assert_allclose(g, g1, rtol=1e-5)
    np.testing.assert_allclose(var, var1, rtol=1e-4)


def _rank_owned_bf(rank, world, port, q):
    import sys
    here = os.path.dirname(os.path.abspath(__file__))
    root = os.path.dirname(here)
    for d in (os.path.join(root, "openmbir-tem_gb300"), os.path.join(root, "oracle"), here):
        sys.path.insert(0, d)
    import torch.distributed as dist
    import mbir
    import shard
    from conftest import bf_case, bf_params
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=world)
    try:
        y, ang, th = bf_case(n_t=16)
        p = bf_params(mbir, th, outer_iterations=BF_OUTER)
        be = shard.OwnedSlabBackend.make(mbir, p, y, ang, world, rank)
        try:
            (y0, y1), hist = shard.run_sharded_bf(dist, be, BF_OUTER)
            vol = shard.gather_volume(dist, be, y0, y1)
            if rank == 0:
                q.put((vol, be.e.nuisance(), np.array(hist)))
        finally:
            be.close()
    finally:
        dist.destroy_process_group()


def test_two_owned_slab_ranks_bright_field_match_one_engine(lib_built):
    """Bright-field NHICD calls on ranks that hold only their slab, halo planes and detector
    rows: the run ends where one engine holding the whole series ends."""
    import multiprocessing as mp
    mbir = lib_built
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_owned_bf, args=(r, 2, port, q)) for r in range(2)]
    for pr in procs:
        pr.start()
    vol, (g, off, var), hist = q.get(timeout=300)
    for pr in procs:
        pr.join(timeout=120)
        assert pr.exitcode == 0
    y, ang, th = bf_case(n_t=16)
    with mbir.Engine(bf_params(mbir, th, outer_iterations=BF_OUTER)) as e:
        e.set_sinogram(y, ang)
        e.prepare()
        first = e.sweep(0, 0)
        np.testing.assert_array_equal(hist[0][2:], first[2:])
    with mbir.Engine(bf_params(mbir, th, outer_iterations=BF_OUTER)) as e:
        e.set_sinogram(y, ang)
        e.run()
        ref = e.volume()
        _, off1, var1 = e.nuisance()
    r = float(np.linalg.norm(vol.astype(np.float64) - ref) / np.linalg.norm(ref))
    assert r <= 1e-4, r
    np.testing.assert_allclose(off, off1, rtol=1e-5)
    np.testing.assert_allclose(var, var1, rtol=1e-4)
