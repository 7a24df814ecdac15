"""The N>1 path of bench.py on CPU (gloo, world size 2): ranks draw disjoint
cells and the job time is the slowest rank's."""

import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    from mpmc_hnu_gb300 import synth

    ncell = 64
    mix, offset, p, t, z, n_near = bench.base_cells(6, ncell, 0.0, rank, synth)
    slowest = bench.max_over_ranks(1.0 + rank, world, "cpu")
    out.put((rank, offset, p.tolist(), slowest))
    dist.barrier()
    dist.destroy_process_group()


def test_two_ranks_draw_disjoint_cells_and_report_the_slowest():
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
    for pr in procs:
        pr.start()
    got = [out.get(timeout=120) for _ in procs]
    for pr in procs:
        pr.join(timeout=120)
        assert pr.exitcode == 0
    got.sort()
    (r0, off0, p0, s0), (r1, off1, p1, s1) = got
    assert off0 != off1
    assert not np.intersect1d(np.array(p0), np.array(p1)).size  # different cells
    assert s0 == s1 == 2.0
