"""The benchmarked workloads at their full sizes, checked through properties that
do not depend on size (the oracle is too slow for them; the small cases are
compared with it bit for bit elsewhere):

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


def test_headline_size_laws_and_conservation(dsm_mod):
    e = _headline(dsm_mod)
    e.init_equilibrium()
    ev = e.advance(100.0)
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


def test_polydisperse_size_classes_full_size(dsm_mod):
    n = 262144
    rng = np.random.default_rng(7)
    s2 = math.log(1.5)
    nkc = np.clip(np.round(np.exp(rng.normal(math.log(150.0) - s2 / 2, math.sqrt(s2), size=n))), 10, 2000)
    nkc = nkc.astype(np.int32)
    e = dsm_mod.Ensemble(nk=int(nkc.max()), n_chains=n, nk_chain=nkc, eq_type=1, sync_dt=1.0, t_end=1.0e6, corr_p=64,
                         corr_m=8, seed=7)
    e.init_equilibrium()
    e.autotune(1.0)
    assert len(e.schedule()) >= 3                    # size classes and the overflow launch
    e.advance(6.0)
    heads, qn, _ = e.get_chains()
    ext = e.get_ext()
    assert np.all(ext["stall"] == 0)
    assert np.all(qn[:, :, 3].sum(axis=1) == nkc)
    assert np.all(heads["Z"] <= nkc)


def test_shear_startup_full_size(dsm_mod):
    """4 x 32768 chains, N_K=100, shear at Wi 1, 10, 100 advanced together
    (dsm_advance_batch), 500 tau_K: Kuhn steps conserved, no stalls, and the
    shear stress grows in magnitude with the Weissenberg number (stress
    -sum 3 Q_x Q_y / N, ensemble_kernel.cu:504-538)."""
    tau_d = dsm_mod.pcd(1.0, 100)["tau_d"]
    wis = (1.0, 10.0, 100.0)
    ens = [dsm_mod.Ensemble(nk=100, n_chains=32768, kappa=(0.0, wi / tau_d, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0),
                            sync_dt=500.0, t_end=5.0e5, seed=4, stream=k) for k, wi in enumerate(wis)]
    for e in ens:
        e.init_equilibrium()
    ev = dsm_mod.advance_batch(ens, 500.0)
    assert np.all(np.asarray(ev) > 0)
    sxy = [e.stress()[0][3] for e in ens]
    assert sxy[2] < sxy[1] < 0.0 and abs(sxy[2]) > 5 * abs(sxy[1])
    for e in ens:
        heads, qn, _ = e.get_chains()
        assert np.all(e.get_ext()["stall"] == 0)
        assert np.all(qn[:, :, 3].sum(axis=1) == 100)
