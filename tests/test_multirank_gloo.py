"""Multi-rank host logic on CPU (gloo, world_size 2).

The engine ships replicas on multi-GPU nodes (one independent system per
GPU).  The contracted-tuple space is still partitioned the reference's way
(loop_size, gam_2_OMP.f:1080-1095), so splitting one system across ranks
is a host range assignment plus one sum of the Fock partials.  This test
runs that split with the oracle on two gloo ranks and checks it against the
single-process result, and checks bench.py's max-over-ranks timing reducer.
"""
from __future__ import annotations

import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, ne, np_, out_dir):
    import torch
    import torch.distributed as dist
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    sys.path.insert(0, ROOT)
    import oracle as O
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    rng = np.random.default_rng(7)
    gee = rng.standard_normal(ne ** 4)
    g2s = rng.standard_normal(ne ** 4 * np_ ** 2)
    DE = np.ascontiguousarray(rng.standard_normal((ne, ne)).ravel(order="F"))
    DP = np.ascontiguousarray(rng.standard_normal((np_, np_)).ravel(order="F"))
    L = O.lib()
    ng4 = ne ** 8 * np_ ** 2
    a, b = np.zeros(1, np.int64), np.zeros(1, np.int64)
    L.orc_loop_size(0, ng4 - 1, world, rank, O.ptr(a), O.ptr(b))
    fe, fp, E = np.zeros(ne * ne), np.zeros(np_ * np_), np.zeros(1)
    L.orc_gam4_dscf_range(ne, np_, O.ptr(gee), O.ptr(g2s), O.ptr(DE), O.ptr(DP),
                          int(a[0]), int(b[0]) + 1, O.ptr(fe), O.ptr(fp), O.ptr(E))
    t = torch.tensor(np.concatenate([fe, fp, E]))
    dist.all_reduce(t)
    tmax = bench.replica_time(dist, world, float(rank + 1))
    if rank == 0:
        np.save(os.path.join(out_dir, "sum.npy"), t.numpy())
        np.save(os.path.join(out_dir, "tmax.npy"), np.array([tmax]))
    dist.destroy_process_group()


def test_two_rank_partition_equals_single_process(orc, tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ne, np_ = 3, 2
    mp.start_processes(_worker, args=(2, _free_port(), ne, np_, str(tmp_path)), nprocs=2,
                       join=True, start_method="spawn")
    got = np.load(tmp_path / "sum.npy")
    rng = np.random.default_rng(7)
    gee = rng.standard_normal(ne ** 4)
    g2s = rng.standard_normal(ne ** 4 * np_ ** 2)
    DE = np.ascontiguousarray(rng.standard_normal((ne, ne)).ravel(order="F"))
    DP = np.ascontiguousarray(rng.standard_normal((np_, np_)).ravel(order="F"))
    L, O = orc.lib(), orc
    fe, fp, E = np.zeros(ne * ne), np.zeros(np_ * np_), np.zeros(1)
    L.orc_gam4_dscf_range(ne, np_, O.ptr(gee), O.ptr(g2s), O.ptr(DE), O.ptr(DP), 0,
                          ne ** 8 * np_ ** 2, O.ptr(fe), O.ptr(fp), O.ptr(E))
    ref = np.concatenate([fe, fp, E])
    np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max())
    assert float(np.load(tmp_path / "tmax.npy")[0]) == 2.0
