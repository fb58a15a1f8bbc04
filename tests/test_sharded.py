"""Sharding one ensemble over ranks (world_size 2, gloo on CPU): per-rank chain
states equal the matching chains of one unsharded run, and the all-reduced
G(t) and stress equal the unsharded ones.  The ranks use the oracle as their
simulator (no GPU here); the sharding and reduction code is the product's
(gpu_dsm_gb300.sharded), and the kernels key their random streams by global
chain id exactly as the oracle does (test_gpu_parity checks the kernels)."""
import os

import numpy as np
import pytest
import torch.multiprocessing as mp

N, NK, T_END = 96, 20, 60.0
SPEC = dict(nk=NK, seed=5, corr=True, sync_dt=1.0, t_end=T_END, corr_p=16, corr_m=2)
SHEAR = dict(nk=NK, seed=6, kappa=(0.0, 5e-3, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0))


def _rank(rank, world, port, out):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from oracle import oracle as orc
    from gpu_dsm_gb300 import sharded

    off, cnt = sharded.shard(N, rank, world)
    o = orc.Oracle(n_chains=cnt, chain_offset=off, threads=1, **SPEC)
    o.init_equilibrium()
    o.run(T_END)
    t, g = sharded.sharded_gt(o, n_total=N, p=16, m=2, sync_dt=1.0, t_end=T_END)
    f = orc.Oracle(n_chains=cnt, chain_offset=off, threads=1, **SHEAR)
    f.init_equilibrium()
    f.run(20.0)
    s, c = sharded.sharded_stress(f)
    st = o.get_state()
    out.put((rank, off, cnt, st["Z"], st["hash"], t, g, s, c))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_shards_equal_one_run(oracle_mod):
    import gpu_dsm_gb300.sharded as sharded

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = sorted(q.get(timeout=300) for _ in range(2))
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    one = oracle_mod.Oracle(n_chains=N, **SPEC)
    one.init_equilibrium()
    one.run(T_END)
    st = one.get_state()
    gsum, _ = one.gt_raw()
    t1, g1 = sharded.gt_points(np.asarray(gsum), n_total=N, p=16, m=2, sync_dt=1.0, t_end=T_END, msd=False)
    for rank, off, cnt, Z, h, t, g, s, c in res:
        assert np.array_equal(Z, st["Z"][off:off + cnt]) and np.array_equal(h, st["hash"][off:off + cnt])
        assert np.array_equal(t, t1)
        assert np.allclose(g, g1, rtol=1e-6, atol=0.0)
    f = oracle_mod.Oracle(n_chains=N, **SHEAR)
    f.init_equilibrium()
    f.run(20.0)
    s1, c1 = f.stress()
    assert res[0][8] == c1 and np.allclose(res[0][7], s1[:8], rtol=1e-6)


@pytest.mark.parametrize("n,world", [(10, 3), (7, 2), (96, 4)])
def test_shard_partition(n, world):
    from gpu_dsm_gb300.sharded import shard

    parts = [shard(n, r, world) for r in range(world)]
    assert sum(c for _, c in parts) == n
    assert all(parts[i][0] + parts[i][1] == parts[i + 1][0] for i in range(world - 1))
