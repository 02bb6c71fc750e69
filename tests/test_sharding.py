"""
Multi-rank sharding of observation points (CPU, gloo, world_size 2): each
rank computes its shard with the CPU oracle and the gathered result equals
the single-process result bitwise (every point's sum is independent).
"""

import os
import socket

import numpy as np
import numpy.testing as npt
import pytest

from harmonica_gb300.sharding import shard_bounds


def test_shard_bounds_cover_everything():
    for n in (0, 1, 7, 100, 101):
        for world in (1, 2, 3, 8):
            spans = [shard_bounds(n, r, world) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(spans, spans[1:]))
            sizes = [h - l for l, h in spans]
            assert max(sizes) - min(sizes) <= 1


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out_path):
    import torch.distributed as dist

    from harmonica_gb300.sharding import forward_sharded
    from oracle import prism_oracle

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    rng = np.random.default_rng(0)
    prisms = np.column_stack([rng.uniform(-1e3, 0, 50), rng.uniform(10, 1e3, 50),
                              rng.uniform(-1e3, 0, 50), rng.uniform(10, 1e3, 50),
                              rng.uniform(-900, -500, 50), rng.uniform(-400, -10, 50)])
    rho = rng.uniform(-300, 300, 50)
    coords = tuple(rng.uniform(-2e3, 2e3, 37) for _ in range(2)) + (100.0,)  # broadcast
    full = forward_sharded(coords, lambda c: prism_oracle.prism_gravity(c, prisms, rho, "g_z",
                                                                       n_threads=1),
                           rank, world)
    if rank == 0:
        np.save(out_path, full)
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_gloo_sharding_matches_single_process(tmp_path, oracle):
    import torch.multiprocessing as mp

    out = str(tmp_path / "full.npy")
    mp.start_processes(_worker, args=(2, _free_port(), out), nprocs=2, start_method="spawn")
    full = np.load(out)
    rng = np.random.default_rng(0)
    prisms = np.column_stack([rng.uniform(-1e3, 0, 50), rng.uniform(10, 1e3, 50),
                              rng.uniform(-1e3, 0, 50), rng.uniform(10, 1e3, 50),
                              rng.uniform(-900, -500, 50), rng.uniform(-400, -10, 50)])
    rho = rng.uniform(-300, 300, 50)
    coords = tuple(rng.uniform(-2e3, 2e3, 37) for _ in range(2)) + (np.full(37, 100.0),)
    npt.assert_array_equal(full, oracle.prism_gravity(coords, prisms, rho, "g_z", n_threads=1))


def _tesseroid_case():
    rng = np.random.default_rng(5)
    r0 = 6371008.8
    w = rng.uniform(-10, 8, 30)
    s = rng.uniform(-10, 8, 30)
    tess = np.column_stack([w, w + rng.uniform(0.5, 2, 30), s, s + rng.uniform(0.5, 2, 30),
                            np.full(30, r0 - 3e4), r0 - rng.uniform(0, 1e3, 30)])
    rho = rng.uniform(2000, 3000, 30)
    coords = (rng.uniform(-12, 12, 41), rng.uniform(-12, 12, 41), r0 + rng.uniform(1e3, 5e4, 41))
    return coords, tess, rho


def _tesseroid_worker(rank, world, port, out_path):
    import torch.distributed as dist

    from harmonica_gb300.sharding import forward_sharded
    from oracle import tesseroid_oracle

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    coords, tess, rho = _tesseroid_case()
    full = forward_sharded(
        coords,
        lambda c: tesseroid_oracle.tesseroid_gravity(c, tess, rho, "g_z", parallel=False),
        rank, world)
    if rank == 0:
        np.save(out_path, full)
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_gloo_sharding_tesseroids(tmp_path):
    """The tesseroid forward shards the same way (points independent): two
    gloo ranks with the tesseroid oracle as the per-shard compute."""
    import torch.multiprocessing as mp

    from oracle import tesseroid_oracle

    out = str(tmp_path / "full_tess.npy")
    mp.start_processes(_tesseroid_worker, args=(2, _free_port(), out), nprocs=2,
                       start_method="spawn")
    coords, tess, rho = _tesseroid_case()
    npt.assert_array_equal(np.load(out),
                           tesseroid_oracle.tesseroid_gravity(coords, tess, rho, "g_z",
                                                              parallel=False))
