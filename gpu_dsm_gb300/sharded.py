"""One ensemble sharded over GPUs (one process per GPU, torch.distributed).

Chains are independent: rank r simulates the contiguous range
[offset_r, offset_r + n_r) of the global ensemble, with every random stream
keyed by the global chain id (``chain_offset``), so each chain's trajectory is
the one it has in a single-GPU run.  The only exchange is at output time: the
correlator sums (sum over chains of C/count per lag) and the stress sums are
added over ranks with one all-reduce each, then normalised by the global
chain count, which gives the single-GPU G(t) / MSD(t) and stress
(the reduction the reference does over call blocks on one GPU,
common/ensemble.cu:289-339, common/ensemble_call_block.cu:452-505).

The reduction logic works on any per-rank ensemble object with ``gt_raw()``
and ``stress()`` of the shapes ``Ensemble`` returns; the tests drive it with
CPU ranks (gloo).
"""
from __future__ import annotations

import math

import numpy as np


def shard(n_total: int, rank: int, world: int):
    """Contiguous partition: (offset, count) of rank's chains."""
    base, extra = divmod(n_total, world)
    count = base + (1 if rank < extra else 0)
    offset = rank * base + min(rank, extra)
    return offset, count


def _allreduce(x: np.ndarray, group=None) -> np.ndarray:
    import torch
    import torch.distributed as dist

    t = torch.from_numpy(np.ascontiguousarray(x, np.float64))
    if dist.get_backend(group) == "nccl":  # NCCL reduces device tensors
        d = t.cuda()
        dist.all_reduce(d, op=dist.ReduceOp.SUM, group=group)
        return d.cpu().numpy()
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return t.numpy()


def gt_points(gsum: np.ndarray, *, n_total: int, p: int, m: int, sync_dt: float, t_end: float, msd: bool):
    """G(t) (or MSD(t)) points of summed raw correlator sums, in the order and
    count gpu_Gt_PCS writes them (common/ensemble.cu:298-335, correlator.cu:146-187)."""
    L = gsum.shape[0]
    dmin = p // m
    npts = p + (L - 1) * (p - dmin)
    actual = npts - p + int(math.floor(t_end / (sync_dt * m ** (L - 1))))
    actual = max(0, min(actual, npts))
    inv = 1.0 / ((1.0 if msd else 3.0) * n_total)
    t, g = [], []
    for k in range(L):
        for j in range(0 if k == 0 else dmin, p):
            if len(t) >= actual:
                break
            t.append(float(j * m ** k))
            g.append(gsum[k, j] * inv)
    return np.array(t, np.float32), np.array(g, np.float32)


def sharded_gt(ens, *, n_total: int, p: int, m: int, sync_dt: float, t_end: float, msd: bool = False, group=None):
    """Global G(t) from per-rank raw sums: one all-reduce."""
    gsum, _ = ens.gt_raw()
    total = _allreduce(np.asarray(gsum, np.float64), group).reshape(np.shape(gsum))
    return gt_points(total, n_total=n_total, p=p, m=m, sync_dt=sync_dt, t_end=t_end, msd=msd)


def sharded_stress(ens, group=None):
    """Global stress average over non-stalled chains: all-reduce of the
    count-weighted sums and the counts."""
    avg, count = ens.stress()
    a = np.asarray(avg, np.float64)[:8]
    total = _allreduce(np.concatenate([a * count, [float(count)]]), group)
    c = total[8]
    return (total[:8] / c if c > 0 else total[:8]), int(round(c))
