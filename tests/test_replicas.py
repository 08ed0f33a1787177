"""Replicas (the multi-GPU form): two gloo ranks on CPU, each solving its own shard of independent problems with the
oracle, then meeting only for the barrier and the max / sum reductions bench.py reports (no data-path collective)."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    import oracle
    from slepc_gb300 import matgen
    from slepc_gb300.replicas import Replicas

    rep = Replicas(backend="gloo")
    problems = [(n, 100 + n) for n in (200, 300, 400, 500, 600)]
    mine = rep.shard(problems)
    rep.barrier()
    conv = 0
    for n, seed in mine:
        csr = matgen.laplacian_2d_randdiag(n, seed)
        r = oracle.solve(*csr, hermitian=True, which="LM", nev=3, ncv=16, tol=1e-10,
                         v0=matgen.start_vector(len(csr[0]) - 1, seed))
        conv += 3 if (r.reason == 1 and r.nconv >= 3) else 0
    rep.barrier()
    out[rank] = (len(mine), rep.sum(conv), rep.max(float(rank + 1)), rep.world)
    rep.close()


@pytest.mark.timeout(300)
def test_replicas_gloo_two_ranks():
    import oracle

    oracle.build()  # before the workers start
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_worker, args=(2, _free_port(), out), nprocs=2, start_method="spawn", join=True)
    assert sorted(out.keys()) == [0, 1]
    assert out[0][0] + out[1][0] == 5 and abs(out[0][0] - out[1][0]) <= 1  # round-robin shards
    assert out[0][1] == out[1][1] == 15.0  # every problem converged, summed over ranks
    assert out[0][2] == out[1][2] == 2.0  # max over ranks
    assert out[0][3] == out[1][3] == 2


def test_replicas_single_process_is_identity():
    from slepc_gb300.replicas import Replicas

    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        os.environ.pop(k, None)
    rep = Replicas()
    assert rep.world == 1 and rep.shard([1, 2, 3]) == [1, 2, 3]
    assert rep.max(2.5) == 2.5 and rep.sum(3.0) == 3.0
    rep.barrier()
    rep.close()
