"""Replica distribution across processes (host logic of the multi-GPU mode), on CPU with gloo."""
import os

import numpy as np
import pytest

from atomnn_gb300 import replicas


def test_shard_covers_every_structure_once():
    for n in (0, 1, 7, 512, 513):
        for world in (1, 2, 3, 8):
            seen = []
            for r in range(world):
                off, cnt = replicas.shard(n, r, world)
                seen.extend(range(off, off + cnt))
            assert seen == list(range(n))


def _worker(rank, world, port, potfile, out):
    import torch.distributed as dist
    from atomnn_gb300 import workloads as W
    from oracle import pyoracle
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world)
    strucs = W.make_structures("mixed512", seed=3, count=7, sizes=[16, 20, 24, 18, 30, 22, 26])
    off, cnt = replicas.shard(len(strucs), rank, world)
    orc = pyoracle.OracleNNP(potfile)
    local = [orc.compute(s.posn, s.species, s.cell, force=False)[0] for s in strucs[off:off + cnt]]
    allres = replicas.gather_results(local)
    if rank == 0:
        np.save(out, np.array(allres))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_gloo_replicas(oracle_lib, pot_mixed, tmp_path):
    import socket
    import torch.multiprocessing as tmp
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    out = str(tmp_path / "e.npy")
    tmp.spawn(_worker, args=(2, port, pot_mixed, out), nprocs=2, join=True)
    from atomnn_gb300 import workloads as W
    strucs = W.make_structures("mixed512", seed=3, count=7, sizes=[16, 20, 24, 18, 30, 22, 26])
    orc = oracle_lib.OracleNNP(pot_mixed)
    serial = [orc.compute(x.posn, x.species, x.cell, force=False)[0] for x in strucs]
    np.testing.assert_allclose(np.load(out), serial, rtol=0, atol=1e-12)
