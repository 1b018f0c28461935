"""Column sharding over two gloo ranks on CPU: the gathered outputs equal a
single-process run column for column (the oracle stands in for each rank's
GPU)."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from socrates_gb300.shard import column_range


def test_column_range_partitions():
    for n in (0, 1, 7, 37, 1000):
        for world in (1, 2, 3, 8):
            spans = [column_range(r, world, n) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == n
            assert all(spans[i][1] == spans[i + 1][0] for i in range(world - 1))
            sizes = [b - a for a, b in spans]
            assert max(sizes) - min(sizes) <= 1


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, results):
    import sys
    from pathlib import Path
    root = Path(__file__).resolve().parent.parent
    for p in (root, root / "oracle", root / "tests" / "golden"):
        sys.path.insert(0, str(p))
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import oracle as O
    from socrates_gb300 import synth
    from socrates_gb300 import radiance as R
    from socrates_gb300.shard import sharded_radiance_calc
    sp, col = synth.config1(37, 30, seed=41)
    out = sharded_radiance_calc(R.lw_noscat_control(), sp, col,
                                run=lambda c, s, cl, mc: O.radiance_calc(c, s, cl, mc))
    if rank == 0:
        results.put({k: v for k, v in out.items()})
    dist.barrier()
    dist.destroy_process_group()


def test_two_ranks_gather_equals_single_run():
    import oracle as O
    from socrates_gb300 import synth
    from socrates_gb300 import radiance as R
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = q.get(timeout=300)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    sp, col = synth.config1(37, 30, seed=41)
    ref = O.radiance_calc(R.lw_noscat_control(), sp, col)
    for k in ref:
        np.testing.assert_array_equal(got[k], ref[k], err_msg=k)
