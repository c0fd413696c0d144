"""The multi-process path of bench.py on CPU: two gloo ranks (the launch `torch.distributed.run`
makes, emulated with spawned processes on 127.0.0.1). Each rank of the GPU arm runs its own
independent system; the ranks exchange a barrier and the largest elapsed time, and the reported
value is the units all ranks processed divided by that time. The reference arm runs on rank 0
alone; the other ranks leave without work."""

import os
import pathlib
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
mp = pytest.importorskip("torch.multiprocessing")

REPO = pathlib.Path(__file__).resolve().parents[1]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    # CPU ranks even where a GPU is visible (gloo, as the two-rank test of the host logic)
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), CUDA_VISIBLE_DEVICES="")
    sys.path.insert(0, str(REPO))
    import bench
    r, w, local = bench.dist_init()
    import torch.distributed as dist
    assert dist.get_backend() == "gloo"
    bench.barrier(w)
    # rank k took (k + 1) ms for its steps: the slowest rank sets the whole job's time
    ms_max = bench.max_over_ranks(float(r + 1), w)
    steps = 100
    value = steps / (ms_max / 1e3) * w  # as run_gb300 reports it: every rank's steps
    # the reference arm: rank 0 alone does the work
    args = type("A", (), {"workload": "lj_fcc_1m"})()
    ran = bench.run_reference(args) if r != 0 else "skipped"
    out.put((r, w, ms_max, value, ran))
    dist.destroy_process_group()


def test_two_gloo_ranks_share_the_slowest_time():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(k, 2, port, q)) for k in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[0] for r in res] == [0, 1]
    assert all(r[1] == 2 for r in res)
    assert all(r[2] == 2.0 for r in res)          # max over ranks of (1, 2) ms
    assert all(abs(r[3] - 100000.0) < 1e-6 for r in res)  # 2 x 100 steps / 2 ms
    assert res[1][4] is None                      # rank 1 of the reference arm: no work
