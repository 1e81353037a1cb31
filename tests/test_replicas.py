"""Replica aggregation of the multi-GPU path, exercised with world_size-2 gloo ranks on
the CPU: throughput = units of all ranks / slowest rank's time."""

import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, ws, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(ws), LOCAL_RANK=str(rank))
    from tatva_gb300 import replicas

    replicas.init("gloo")
    assert replicas.world() == (ws, rank, rank)
    replicas.barrier()
    units = 1000.0 * (rank + 1)      # each replica processed its own batch
    secs = 0.5 + 0.25 * rank         # the slower rank bounds the job
    out[rank] = (replicas.max_over_ranks(secs), replicas.sum_over_ranks(units),
                 replicas.aggregate_throughput(units, secs))
    replicas.barrier()
    import torch.distributed as dist

    dist.destroy_process_group()


def test_two_gloo_replicas_aggregate():
    ws, port = 2, _free_port()
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_rank_main, args=(ws, port, out), nprocs=ws, start_method="spawn",
                       join=True)
    for r in range(ws):
        mx, sm, thr = out[r]
        assert mx == pytest.approx(0.75) and sm == pytest.approx(3000.0)
        assert thr == pytest.approx(3000.0 / 0.75)


def test_single_process_is_identity():
    from tatva_gb300 import replicas

    assert replicas.max_over_ranks(2.0) == 2.0
    assert replicas.aggregate_throughput(10.0, 2.0) == 5.0
