"""Synthetic catalogue generators, and the replica (multi-process) timing helpers of bench.py on
CPU with the gloo backend, world size 2."""
import os
import socket
import sys

import numpy as np
import pytest

from capow_gb300 import synth

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_uniform_is_seeded_and_inside_box():
    a = synth.uniform(1000, L=500.0, seed=1)
    b = synth.uniform(1000, L=500.0, seed=1)
    for u, v in zip(a, b):
        assert np.array_equal(u, v)
    for c in a[:3]:
        assert c.min() >= 0.0 and c.max() < 500.0
    assert abs(np.std(np.concatenate(a[3:])) - 300.0) < 15.0


def test_zeldovich_displacement_and_bounds():
    L, mesh, ns = 1000.0, 64, 32
    x, y, z, vx, vy, vz = synth.zeldovich(ns, L=L, mesh=mesh, rms_cells=1.5, seed=2)
    assert x.dtype == np.float32 and len(x) == ns ** 3
    for c in (x, y, z):
        assert c.min() >= 0.0 and c.max() < np.float32(L)
    # displacement from the lattice, modulo the box: rms 3-D = 1.5 mesh cells
    q = (np.arange(ns) + 0.5) * (L / ns)
    qx, qy, qz = np.meshgrid(q, q, q, indexing="ij")
    d = [((c.astype(np.float64) - g.ravel() + L / 2) % L) - L / 2 for c, g in ((x, qx), (y, qy), (z, qz))]
    rms = np.sqrt(np.mean(d[0] ** 2 + d[1] ** 2 + d[2] ** 2))
    assert abs(rms - 1.5 * L / mesh) < 0.01 * L / mesh
    # velocities: 80 * Psi + N(0, 150)
    v = vx.astype(np.float64) - 80.0 * d[0]
    assert abs(np.std(v) - 150.0) < 5.0


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    bench.barrier(world)
    m = bench.max_over_ranks(world, float(10 + rank), "cpu")
    dist.destroy_process_group()
    q.put((rank, m))


def test_replicas_take_max_over_ranks_gloo():
    import multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    got = dict(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
    assert got == {0: 11.0, 1: 11.0}


def test_algorithmic_bytes_formula():
    import importlib

    sys.path.insert(0, ROOT)
    bench = importlib.import_module("bench")
    ng, nc = 512 ** 3, 512 * 512 * 257
    b = bench.algorithmic_bytes(256 ** 3, ng, nc, 4, 16, 4, 8)
    assert abs(b / 1e9 - 8.875) < 0.01  # the headline workload's algorithmic bytes per evaluation
