"""The multi-GPU path of bench.py is replicas only (one independent network per rank, no
collective on the data path): its host logic -- barriers, the max of the per-rank times and the
sum of the per-rank events -- runs here as world_size-2 gloo process groups on the CPU."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

from conftest import ROOT


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, ws, port, out):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "WORLD_SIZE": str(ws), "LOCAL_RANK": str(rank)})
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    got_ws, got_rank, _ = bench._dist()
    bench._barrier(ws)
    ms = 10.0 + rank * 5.0          # per-rank timed region
    events = 1000.0 * (rank + 1)    # per-rank events
    out[rank] = (got_ws, got_rank, bench._max_over_ranks(ms, ws), bench._sum_over_ranks(events, ws))
    bench._barrier(ws)
    dist.destroy_process_group()


def test_replica_reductions_world_size_2():
    port = _free_port()
    with mp.get_context("spawn").Manager() as mgr:
        out = mgr.dict()
        mp.spawn(_worker, args=(2, port, out), nprocs=2, join=True)
        res = dict(out)
    for rank in (0, 1):
        ws, r, ms, ev = res[rank]
        assert (ws, r) == (2, rank)
        assert ms == 15.0            # the slowest rank's time
        assert ev == 3000.0          # every rank's events
    # whole-job value = all ranks' events over the slowest rank's time
    assert res[0][3] / (res[0][2] / 1e3) == pytest.approx(200000.0)


def _ref_worker(rank, ws, port, out):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "WORLD_SIZE": str(ws), "LOCAL_RANK": str(rank)})
    sys.path.insert(0, ROOT)
    import bench

    class A:
        steps, warmup, gpus = 1, 1, ws
    if rank != 0:
        out[rank] = bench.reference_arm(A())  # other ranks exit 0 without work


def test_reference_arm_other_ranks_do_no_work():
    with mp.get_context("spawn").Manager() as mgr:
        out = mgr.dict()
        mp.spawn(_ref_worker, args=(2, _free_port(), out), nprocs=2, join=True)
        assert dict(out)[1] == 0
