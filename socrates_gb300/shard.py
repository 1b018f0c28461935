"""Column sharding over ranks.

Columns are independent on the two-stream path, so a batch splits into
contiguous column windows, one per rank (one GPU each), with no exchange
during the solve.  The only collective is the host-side gather of the
output slabs, over torch.distributed (nccl between GPUs, gloo on CPU).
"""
from __future__ import annotations

import numpy as np

from . import synth


def column_range(rank: int, world: int, n: int) -> tuple[int, int]:
    """[start, stop) of rank's contiguous window of n columns (balanced)."""
    base, extra = divmod(n, world)
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def sharded_radiance_calc(control, spectrum, col, mcica=None, run=None, group=None) -> dict:
    """radiance_calc over all ranks of `group`: each rank solves its own
    column window with `run` (default: the CUDA path of this process's
    device) and every rank receives the whole batch's outputs."""
    import torch.distributed as dist
    from dataclasses import replace
    if run is None:
        from .radiance import radiance_calc as run
    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    c0, c1 = column_range(rank, world, col.n_profile)
    mine = synth.window(col, c0, c1 - c0)
    mc = None
    if mcica is not None:
        sl = slice(c0, c1)
        mc = replace(mcica, c_sub=np.asfortranarray(mcica.c_sub[sl]),
                     n_subcol_cld=np.ascontiguousarray(mcica.n_subcol_cld[sl]),
                     frac_cloudy=np.ascontiguousarray(mcica.frac_cloudy[sl]))
    out = run(control, spectrum, mine, mc) if c1 > c0 else {}
    slabs = [None] * world
    dist.all_gather_object(slabs, (c0, c1, out), group=group)
    full = {}
    for a, b, o in slabs:
        for k, v in o.items():
            if k not in full:
                full[k] = np.zeros((col.n_profile,) + v.shape[1:], order="F")
            full[k][a:b] = v
    return full
