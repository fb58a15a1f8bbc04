"""The benchmarked configurations against the oracle, and every measured
observable against the FP64 transcription.

Config 1 (1024 chains x N_K=25, beta=1, t = 1e4 tau_K, G(t) of sigma_xy with
p=16, m=2, seeds 1, 2, 3) runs in full on the GPU and in the oracle: chain
states bit for bit, G(t) sums within 1e-5.

Error against the FP64 oracle (mode 1): modes 0 (which the GPU reproduces) and
1 draw the same random words, so the GPU's G(t) or stress and the FP64 ones
are estimates on the same trajectories up to the rare chains whose event
sequence a rounding difference changed.  The error is judged against the FP64
estimate's own statistical error sigma (chain-to-chain, per lag or output
time): at most 1 % on every lag resolved to 2 % statistical precision, at most
2 sigma anywhere, at most 1 % of G(lag 0).

The full-size configurations 2-4 are compared chain for chain in
test_gpu_fullsize.py."""
import numpy as np
import pytest

from helpers import assert_bitexact, gpu_state

pytestmark = pytest.mark.gpu


def _fp64_ok(err):
    assert err["rel_resolved"] is None or err["rel_resolved"] <= 0.01, err
    assert err["dev_sigma"] <= 2.0, err
    assert err["rel_scale"] <= 0.01, err


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_config1_in_full(dsm_mod, oracle_mod, seed):
    """Config 1 exactly as stated, GPU against the oracle."""
    kw = dict(nk=25, n_chains=1024, sync_dt=1.0, t_end=1.0e4, corr_p=16, corr_m=2, seed=seed)
    g = dsm_mod.Ensemble(eq_type=1, **kw)
    o = oracle_mod.Oracle(corr=True, **kw)
    g.init_equilibrium()
    o.init_equilibrium()
    ev = g.advance(1.0e4)
    assert ev == o.run(1.0e4)
    assert_bitexact(gpu_state(g), o.get_state(), what=f"config 1 seed {seed}")
    gs, gc = g.gt_raw()
    os_, oc = o.gt_raw()
    assert np.array_equal(gc, oc)
    m = oc > 0
    assert np.max(np.abs(gs[m] - os_[m])) <= 1e-5 * np.abs(os_[m]).max()
    if seed == 1:
        f = oracle_mod.Oracle(corr=True, mode=1, **kw)
        f.init_equilibrium()
        f.run(1.0e4)
        _fp64_ok(oracle_mod.gt_error_vs_fp64(gs, f))


def test_config2_gt_vs_fp64(dsm_mod, oracle_mod):
    """Headline parameters (N_K=200, beta=1, G(t) over xy/yz/xz, p=64, m=8) on 512
    of the headline ensemble's chains (global ids 30000-30511): state bit for bit
    with the oracle, G(t) against the FP64 transcription."""
    kw = dict(nk=200, n_chains=512, sync_dt=1.0, t_end=1.0e7, corr_p=64, corr_m=8, seed=5, chain_offset=30000)
    g = dsm_mod.Ensemble(eq_type=1, **kw)
    o = oracle_mod.Oracle(corr=True, **kw)
    f = oracle_mod.Oracle(corr=True, mode=1, **kw)
    for x in (g, o, f):
        x.init_equilibrium()
    g.advance(500.0)
    o.run(500.0)
    f.run(500.0)
    assert_bitexact(gpu_state(g), o.get_state(), what="config 2 slice")
    gs, gc = g.gt_raw()
    os_, oc = o.gt_raw()
    assert np.array_equal(gc, oc)
    m = oc > 0
    assert np.max(np.abs(gs[m] - os_[m])) <= 1e-5 * np.abs(os_[m]).max()
    # 512 chains resolve no lag to 2 %: the paired deviation in sigma and
    # relative to G(lag 0) carry the comparison
    _fp64_ok(oracle_mod.gt_error_vs_fp64(gs, f))


@pytest.mark.parametrize("wi", [10.0, 100.0])
def test_config4_stress_vs_fp64(dsm_mod, oracle_mod, wi):
    """Shear start-up (N_K=100, kappa_xy = Wi / tau_d) on 512 chains, ten output
    windows of 100 tau_K: GPU state bit for bit with the oracle at every
    output; sigma_xy consistent with the FP64 transcription within three joint
    standard errors (3 sqrt(2) sigma).  Under flow the FP32 and FP64
    trajectories decorrelate within ~1e4 events per chain (every deformation
    rounds differently), so late outputs compare near-independent estimates."""
    tau_d = dsm_mod.pcd(1.0, 100)["tau_d"]
    kap = (0.0, wi / tau_d, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0)
    kw = dict(nk=100, n_chains=512, kappa=kap, seed=4, stream=3, chain_offset=7000)
    g = dsm_mod.Ensemble(sync_dt=100.0, t_end=5.0e5, **kw)
    o = oracle_mod.Oracle(**kw)
    f = oracle_mod.Oracle(mode=1, **kw)
    for x in (g, o, f):
        x.init_equilibrium()
    worst = 0.0
    for w in range(1, 11):
        t = 100.0 * w
        g.advance(t)
        o.run(t)
        f.run(t)
        assert_bitexact(gpu_state(g), o.get_state(), keys=("Z", "QN", "tau", "T", "step", "hash", "stall", "dt_prev"),
                        what=f"shear Wi={wi} t={t}")
        sg, cg = g.stress()
        sf, cf = f.stress()
        assert cg == cf == 512
        st = f.get_state()
        Z = st["Z"]
        q = st["QN"].astype(np.float64)
        idx = np.arange(q.shape[1])[None, :] < Z[:, None]
        per = -3.0 * np.where(idx, q[:, :, 0] * q[:, :, 1] / np.where(idx, q[:, :, 3], 1.0), 0.0).sum(axis=1)
        sig = per.std(ddof=1) / np.sqrt(len(per))
        d = abs(sg[3] - sf[3])
        assert d <= 3.0 * np.sqrt(2.0) * sig, (t, sg[3], sf[3], sig)
        worst = max(worst, d / sig)
    assert worst < 3.0 * np.sqrt(2.0)
