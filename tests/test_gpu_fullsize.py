"""The benchmarked workloads at their full sizes, on the schedules the bench
uses.  Random streams are keyed by the global chain id, so the oracle replays
slices of each full-size ensemble (chain_offset; for the polydisperse melt with
the whole ensemble's N_K list as the partner law) and those chains must equal
the GPU's bit for bit: at 100 tau_K of the headline ensemble, after the
autotuner and a window of the polydisperse melt (slices around the longest
chains and the class boundaries), and at every output of the batched shear
start-up at Wi 0.1, 1, 10, 100.  Size-independent properties are checked over
all chains:

- 65536 chains x N_K=200, beta=1, G(t) p=64 m=8 (the headline ensemble):
  conservation of Kuhn steps per chain, the equilibrium laws after a run
  (Z - 1 ~ Binomial(N_K - 1, 1/(1+beta)), <3 Q_x^2 / N> = 1 over internal
  strands; chain.cu:38-102, detailed_balance.h:44-54), no stalls, G(t)
  positive and decaying at short lags, bit-exact reproducibility, and the
  same chains whether run as one ensemble or as two shards (chain_offset);
- 262144 polydisperse chains (log-normal N_K, mean 150, PDI 1.5, <= 2000)
  in size classes after autotuning: conservation and no stalls;
- shear start-up, 4 x 32768 chains, N_K=100: conservation, no stalls, shear
  stress ordered by the Weissenberg number."""
import math

import numpy as np
import pytest
from scipy import stats

from helpers import assert_bitexact, gpu_state

pytestmark = pytest.mark.gpu

N, NK = 65536, 200


def _headline(dsm_mod, n=N, chain_offset=0):
    return dsm_mod.Ensemble(nk=NK, n_chains=n, beta=1.0, eq_type=1, sync_dt=1.0, t_end=1.0e7, corr_p=64, corr_m=8,
                            seed=5, chain_offset=chain_offset)


def _slices_bitexact(gpu: dict, make_oracle, offsets, width, t, what, keys=None):
    """Run the oracle on chains [off, off + width) of a GPU ensemble and compare."""
    for off in offsets:
        o = make_oracle(off, width)
        o.init_equilibrium()
        o.run(t)
        part = {k: v[off:off + width] for k, v in gpu.items()}
        kw = {} if keys is None else {"keys": keys}
        assert_bitexact(part, o.get_state(), what=f"{what}, chains {off}-{off + width - 1}", **kw)


def test_headline_size_laws_and_conservation(dsm_mod, oracle_mod):
    e = _headline(dsm_mod)
    e.init_equilibrium()
    ev = e.advance(100.0)
    # chain slices of the full ensemble against the oracle, bit for bit
    _slices_bitexact(gpu_state(e), lambda off, w: oracle_mod.Oracle(
        nk=NK, n_chains=w, seed=5, corr=True, sync_dt=1.0, t_end=1.0e7, corr_p=64, corr_m=8, chain_offset=off),
        (0, 16384 + 777, 40000, N - 256), 256, 100.0, "headline ensemble")
    heads, qn, _ = e.get_chains()
    ext = e.get_ext()
    Z = heads["Z"].astype(np.int64)
    assert np.all(ext["stall"] == 0)
    assert np.all(qn[:, :, 3].sum(axis=1) == NK)              # Kuhn steps conserved per chain
    assert Z.min() >= 1 and Z.max() <= NK
    # about 42.6 events per chain per tau_K at N_K=200, beta=1
    assert 0.8 * 42.6 * 100 * N < ev < 1.2 * 42.6 * 100 * N
    # Z law: chi-square goodness of fit against the binomial (bins with >= 50 expected)
    law = stats.binom(NK - 1, 0.5)
    k = np.arange(NK)
    expect = law.pmf(k) * N
    keep = expect >= 50
    obs = np.bincount(Z - 1, minlength=NK)
    lo, hi = k[keep][0], k[keep][-1]
    o = np.concatenate([[obs[:lo].sum()], obs[keep], [obs[hi + 1:].sum()]])
    x = np.concatenate([[expect[:lo].sum()], expect[keep], [expect[hi + 1:].sum()]])
    chi = ((o - x) ** 2 / x).sum()
    assert stats.chi2.sf(chi, len(o) - 1) > 1e-4, chi
    # Q law of the internal strands: 3 Q_x^2 / N ~ chi^2_1, mean 1
    idx = np.arange(NK)[None, :]
    internal = (idx >= 1) & (idx < (Z - 1)[:, None])
    w = 3.0 * qn[:, :, 0][internal].astype(np.float64) ** 2 / qn[:, :, 3][internal]
    assert abs(w.mean() - 1.0) < 5 * math.sqrt(2.0 / w.size)
    # G(t): positive, decaying over the first lags
    t, G = e.gt()
    assert np.all(np.isfinite(G)) and G[0] > 0 and np.all(G[:16] > 0)
    assert np.all(np.diff(G[:16]) <= 0)


def test_headline_size_reproducible_and_shard_invariant(dsm_mod):
    a = _headline(dsm_mod)
    b = _headline(dsm_mod)
    for x in (a, b):
        x.init_equilibrium()
        x.advance(20.0)
    sa = gpu_state(a)
    assert_bitexact(gpu_state(b), sa, what="same seed, same bits")
    # the same ensemble as two shards of 32768 chains (global chain ids)
    half = N // 2
    for off in (0, half):
        s = _headline(dsm_mod, n=half, chain_offset=off)
        s.init_equilibrium()
        s.advance(20.0)
        part = {k: v[off:off + half] for k, v in sa.items()}
        assert_bitexact(gpu_state(s), part, what=f"shard at {off}")


def test_polydisperse_size_classes_full_size(dsm_mod, oracle_mod):
    n = 262144
    rng = np.random.default_rng(7)
    s2 = math.log(1.5)
    nkc = np.clip(np.round(np.exp(rng.normal(math.log(150.0) - s2 / 2, math.sqrt(s2), size=n))), 10, 2000)
    nkc = nkc.astype(np.int32)
    nkmax = int(nkc.max())
    e = dsm_mod.Ensemble(nk=nkmax, n_chains=n, nk_chain=nkc, eq_type=1, sync_dt=1.0, t_end=1.0e6, corr_p=64,
                         corr_m=8, seed=7)
    e.init_equilibrium()
    tuned = e.autotune(1.0)                          # one 1-tau_K window per candidate schedule
    assert len(e.schedule()) >= 3                    # size classes and the overflow launch
    t1 = tuned["candidates"] * 1.0 + 5.0
    e.advance(t1)
    heads, qn, _ = e.get_chains()
    ext = e.get_ext()
    assert np.all(ext["stall"] == 0)
    assert np.all(qn[:, :, 3].sum(axis=1) == nkc)
    assert np.all(heads["Z"] <= nkc)
    # slices around chains of every size class: the longest chains (huge and
    # large classes), the tail of the middle class, the bulk
    order = np.argsort(nkc, kind="stable")
    centres = [int(order[-1]), int(order[-40]), int(order[int(0.995 * n)]), int(order[int(0.95 * n)]),
               int(order[n // 2]), int(order[n // 10])]
    w = 24
    offs = sorted({min(max(0, c - w // 2), n - w) for c in centres})
    _slices_bitexact(gpu_state(e), lambda off, w_: oracle_mod.Oracle(
        nk=nkmax, n_chains=w_, nk_chain=nkc[off:off + w_], partner_nk=nkc, seed=7, corr=True, sync_dt=1.0,
        t_end=1.0e6, corr_p=64, corr_m=8, chain_offset=off), offs, w, t1, "polydisperse melt")


def test_shear_startup_full_size(dsm_mod, oracle_mod):
    """4 x 32768 chains, N_K=100, shear at Wi 0.1, 1, 10, 100 advanced together
    (dsm_advance_batch, as the bench runs them), two 500 tau_K output windows:
    slices of every ensemble equal the oracle at both outputs, Kuhn steps are
    conserved, no chain stalls, and the shear stress grows in magnitude with
    the Weissenberg number (-sum 3 Q_x Q_y / N, ensemble_kernel.cu:504-538)."""
    tau_d = dsm_mod.pcd(1.0, 100)["tau_d"]
    wis = (0.1, 1.0, 10.0, 100.0)
    kaps = [(0.0, wi / tau_d, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0) for wi in wis]
    ens = [dsm_mod.Ensemble(nk=100, n_chains=32768, kappa=kap, sync_dt=500.0, t_end=5.0e5, seed=4, stream=k)
           for k, kap in enumerate(kaps)]
    for e in ens:
        e.init_equilibrium()
    offs, w = (0, 20000, 32768 - 64), 64
    orcs = {(k, off): oracle_mod.Oracle(nk=100, n_chains=w, kappa=kaps[k], seed=4, stream=k, chain_offset=off)
            for k in range(len(ens)) for off in offs}
    for o in orcs.values():
        o.init_equilibrium()
    for t in (500.0, 1000.0):
        ev = dsm_mod.advance_batch(ens, t)
        assert np.all(np.asarray(ev) > 0)
        for k, e in enumerate(ens):
            st = gpu_state(e)
            for off in offs:
                o = orcs[(k, off)]
                o.run(t)
                assert_bitexact({q: v[off:off + w] for q, v in st.items()}, o.get_state(),
                                keys=("Z", "QN", "tau", "T", "step", "hash", "S", "stall", "dt_prev"),
                                what=f"shear Wi={wis[k]} t={t}, chains {off}-{off + w - 1}")
    sxy = [e.stress()[0][3] for e in ens]
    assert sxy[3] < sxy[2] < 0.0 and abs(sxy[3]) > 5 * abs(sxy[2])
    for e in ens:
        heads, qn, _ = e.get_chains()
        assert np.all(e.get_ext()["stall"] == 0)
        assert np.all(qn[:, :, 3].sum(axis=1) == 100)
