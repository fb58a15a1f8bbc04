"""The oracle pinned against the reference: Philox known answers, element-wise
math accuracy, p_cd constants and equilibrium-initialiser statistics of the
compiled reference host code (golden fixtures), the analytic DSM laws, and
stationarity (detailed balance) of the kMC dynamics."""
import json
import math
from pathlib import Path

import numpy as np
import pytest
from scipy import stats

GOLD = Path(__file__).resolve().parent / "golden"
PCD_NAMES = ["alpha", "tau_0", "tau_max", "tau_d", "g", "c1", "cm1", "rcm1c1", "At", "Adt", "Bdt", "normdt"]


def test_philox_known_answers(oracle_mod):
    # Random123 known-answer vectors for philox4x32_10
    kat = [((0, 0, 0, 0), (0, 0), (0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8)),
           ((0xffffffff,) * 4, (0xffffffff,) * 2, (0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd)),
           ((0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344), (0xa4093822, 0x299f31d0),
            (0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1))]
    for ctr, key, want in kat:
        assert tuple(int(v) for v in oracle_mod.philox(ctr, key)) == want


def test_math_accuracy(oracle_mod):
    x = np.linspace(-80, 80, 100001).astype(np.float32)
    y = oracle_mod.math_f(0, x=x)
    assert np.max(np.abs(y - np.exp(x.astype(np.float64))) / np.exp(x.astype(np.float64))) < 2.5e-7
    x = np.exp(np.linspace(-17, 20, 100001)).astype(np.float32)
    y = oracle_mod.math_f(1, x=x)
    ref = np.log(x.astype(np.float64))
    assert np.max(np.abs(y - ref)) < 2.5e-6
    w = np.arange(0, 1 << 24, 97, dtype=np.uint32)
    th = 2 * np.pi * w / 2.0 ** 24
    assert np.max(np.abs(oracle_mod.math_f(3, w=w) - np.sin(th))) < 2e-7
    assert np.max(np.abs(oracle_mod.math_f(4, w=w) - np.cos(th))) < 2e-7
    # Box-Muller output is standard normal
    rng = np.random.default_rng(0)
    ww = rng.integers(0, 2 ** 32, size=2 * 200000, dtype=np.uint32)
    g = oracle_mod.math_f(2, w=ww, n=200000)
    assert abs(g.mean()) < 0.01 and abs(g.var() - 1) < 0.01
    assert stats.kstest(g, "norm").pvalue > 1e-3


def test_pcd_matches_reference(oracle_mod):
    """p_cd fits (pcd_tau.h:32-66): double evaluation vs the reference's float code."""
    d = json.loads((GOLD / "pcd_reference.json").read_text())
    for r in d["rows"]:
        ours, _ = oracle_mod.pcd(r["beta"], r["nk"])
        for k, v in zip(PCD_NAMES, ours):
            assert v == pytest.approx(r[k], rel=1e-5, abs=1e-12), (r["beta"], r["nk"], k)


def test_tau_samplers_match_reference(oracle_mod):
    """Lifetime samplers: quantiles of the float spec vs the reference samplers."""
    d = json.loads((GOLD / "tau_reference.json").read_text())
    u = ((np.arange(200000, dtype=np.uint32) * 2654435761) >> 8).astype(np.float64)
    u = ((u + 1) / 2.0 ** 24).astype(np.float32)
    for r in d["rows"]:
        kind = 0 if r["kind"] == "f_t" else 1
        rate = oracle_mod.tau_samples(r["beta"], r["nk"], kind, 0, u)
        rate64 = oracle_mod.tau_samples(r["beta"], r["nk"], kind, 1, u)
        # float spec vs the double formula: ~1e-7 typically; up to ~2e-3 for the
        # longest CD-created lifetimes, where u*Adt'+Ddt cancels to ~tau_max^(alpha-1)
        # and the float rounding of the constants dominates (same in the reference's
        # float code, gpu_random.cu:143-145)
        err = np.abs(rate - rate64) / rate64
        assert np.median(err) < 1e-6 and err.max() < 3e-3
        # weight of the tau_d spike: g for f_t, (g/tau_d)/normdt for f_d*t (pcd_tau.h:67-82)
        p64, _ = oracle_mod.pcd(r["beta"], r["nk"])
        g, tau_d, normdt = p64[4], p64[3], p64[11]
        w_spike = g if kind == 0 else (g / tau_d) / normdt
        assert np.mean(rate == rate.min()) == pytest.approx(w_spike, abs=0.01)
        tau = np.sort(1.0 / rate)
        # the reference sample's q-quantile must sit at CDF ~ q of our sampler,
        # within the sampling error of a quantile of n reference draws
        for q, v in r["tau_quantiles"].items():
            q = float(q)
            if v >= tau[-1] * (1 - 1e-5):
                continue  # inside the tau_d spike of the law (weight g or g/tau_d/normdt)
            cdf = np.searchsorted(tau, v, side="right") / tau.size
            tol = 5.0 * math.sqrt(q * (1 - q) / r["n"]) + 2e-3
            assert abs(cdf - q) <= tol, (r["beta"], r["nk"], r["kind"], q, cdf)


def _binom_law(nk, beta):
    p = 1.0 / (1.0 + beta)
    return stats.binom(nk - 1, p)


@pytest.mark.parametrize("idx", [0, 1, 2, 3])
def test_init_matches_reference_and_law(oracle_mod, idx):
    """Equilibrium initialiser vs reference chain_init (chain.cu:199-283) and the
    analytic law Z-1 ~ Binomial(NK-1, 1/(1+beta)) (chain.cu:106-117,
    detailed_balance.h:44-54)."""
    g = json.loads((GOLD / "init_reference.json").read_text())["ensembles"][idx]
    nk, beta, n = g["nk"], g["beta"], g["n_chains"]
    o = oracle_mod.Oracle(nk=nk, beta=beta, n_chains=n, seed=17)
    o.init_equilibrium()
    st = o.get_state()
    Z = st["Z"]
    zh = np.bincount(Z, minlength=nk + 1)[: nk + 1]
    ref = np.array(g["z_hist"])
    # two-sample chi-square on Z (bins with enough counts)
    tab = np.vstack([zh, ref])
    keep = tab.sum(axis=0) >= 20
    chi = stats.chi2_contingency(tab[:, keep])
    assert chi.pvalue > 1e-4, chi
    # against the analytic binomial law
    law = _binom_law(nk, beta)
    assert abs(Z.mean() - 1 - law.mean()) < 5 * law.std() / math.sqrt(n)
    # N histogram: two-sample chi-square
    N = np.concatenate([st["QN"][i, : Z[i], 3] for i in range(n)]).astype(int)
    nh = np.bincount(N, minlength=nk + 1)[: nk + 1]
    tab = np.vstack([nh, np.array(g["n_hist"])])
    keep = tab.sum(axis=0) >= 20
    assert stats.chi2_contingency(tab[:, keep]).pvalue > 1e-4
    # Q ~ N(0, N/3) for internal strands: Q^2/N has mean 1 and var 2/3
    q2n = np.concatenate([np.sum(st["QN"][i, 1: Z[i] - 1, :3] ** 2, axis=1) / st["QN"][i, 1: Z[i] - 1, 3]
                          for i in range(n) if Z[i] > 2])
    assert q2n.mean() == pytest.approx(g["q2_over_n_mean"], abs=0.03)
    assert q2n.mean() == pytest.approx(1.0, abs=0.03)
    assert q2n.var() == pytest.approx(2.0 / 3.0, rel=0.06)
    # dangling ends carry no connector; N sums to NK
    ends = np.array([np.abs(st["QN"][i, [0, Z[i] - 1], :3]).max() for i in range(n)])
    assert ends.max() == 0.0 == g["max_abs_end_q"]
    assert all(st["QN"][i, : Z[i], 3].sum() == nk for i in range(n))
    # lifetime rates of the initial entanglements: quantiles vs reference
    rates = np.concatenate([st["tau"][i, : Z[i] - 1] for i in range(n)])
    for q, v in g["rate_quantiles"].items():
        if 0.01 <= float(q) <= 0.6:  # above 1-g all rates equal 1/tau_d
            assert np.quantile(rates, float(q)) == pytest.approx(v, rel=0.06), q


def test_conservation_and_ranges(oracle_mod):
    o = oracle_mod.Oracle(nk=30, n_chains=512, seed=2)
    o.init_equilibrium()
    ev = o.run(300.0)
    st = o.get_state()
    assert ev > 0
    Z = st["Z"]
    for i in range(512):
        N = st["QN"][i, : Z[i], 3]
        assert N.sum() == 30 and N.min() >= 1
        assert np.all(st["QN"][i, [0, Z[i] - 1], :3] == 0)
    assert np.all(st["stall"] == 0)
    assert np.all(st["T"] >= 300 * 2 ** 32)


@pytest.mark.slow
def test_stationarity_detailed_balance(oracle_mod):
    """The kMC dynamics must keep the equilibrium laws stationary (the reference
    builds its rates to satisfy detailed balance): after 3000 tau_K the P(Z),
    N and Q statistics still follow the analytic law."""
    nk, n = 25, 4096
    o = oracle_mod.Oracle(nk=nk, n_chains=n, seed=5)
    o.init_equilibrium()
    o.run(3000.0)
    st = o.get_state()
    Z = st["Z"]
    law = _binom_law(nk, 1.0)
    k = np.arange(0, nk)
    obs = np.bincount(Z - 1, minlength=nk)[:nk]
    exp = law.pmf(k) * n
    keep = exp >= 10
    chi2 = (((obs[keep] - exp[keep]) ** 2) / exp[keep]).sum()
    assert stats.chi2(keep.sum() - 1).sf(chi2) > 1e-4, (obs, exp)
    q2n = np.concatenate([np.sum(st["QN"][i, 1: Z[i] - 1, :3] ** 2, axis=1) / st["QN"][i, 1: Z[i] - 1, 3]
                          for i in range(n) if Z[i] > 2])
    assert q2n.mean() == pytest.approx(1.0, abs=0.04)
    # internal and end strand N: uniform compositions -> E[N] = NK/Z per chain
    meanN = np.array([st["QN"][i, : Z[i], 3].mean() for i in range(n)])
    assert np.allclose(meanN * Z, nk)


def test_fp64_transcription_agrees_statistically(oracle_mod):
    """FP32-mirror arithmetic (fixed-point pick, table rates) vs the literal FP64
    transcription: same event rate per chain per tau and same <Z>."""
    res = {}
    for mode in (0, 1):
        o = oracle_mod.Oracle(nk=25, n_chains=2048, seed=8, mode=mode)
        o.init_equilibrium()
        o.run(50.0)
        ev = o.run(450.0)
        st = o.get_state()
        res[mode] = (ev / 2048 / 400.0, st["Z"].mean())
    assert res[0][0] == pytest.approx(res[1][0], rel=0.01)
    assert res[0][1] == pytest.approx(res[1][1], abs=0.15)
    assert res[0][0] == pytest.approx(7.0, rel=0.05)  # <sum W> at NK=25, beta=1


def test_flow_shear_stress_sign(oracle_mod):
    """Start-up of shear: sigma_xy grows from 0 with the sign of kappa_xy
    (stress = -3 sum QxQy/N, ensemble_kernel.cu:523-528)."""
    kap = (0.0, 1e-2, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0)
    o = oracle_mod.Oracle(nk=25, n_chains=2048, seed=3, kappa=kap)
    o.init_equilibrium()
    s0, _ = o.stress()
    o.run(20.0)
    s1, c = o.stress()
    assert c == 2048
    assert s1[3] < s0[3] - 0.05  # sxy = -3<QxQy/N> becomes negative for kappa_xy > 0


@pytest.mark.parametrize("p,m,levels,n", [(16, 2, 6, 1000), (64, 8, 3, 5000)])
def test_correlator_matches_bruteforce(oracle_mod, p, m, levels, n):
    """Multi-tau correlator (eq_ensemble_kernel.cu:133-227): level k holds block
    averages of m^k consecutive samples; lag j of level k (j >= p/m for k > 0)
    accumulates sum_i y_k(i) . y_k(i-j) over the last p values.  Checked
    against the O(n^2) definition on a random series."""
    rng = np.random.default_rng(1)
    x = rng.standard_normal((n, 3)).cumsum(axis=0) * 0.1
    acc, nins = oracle_mod.corr_series(x, p, m, levels)
    dmin = p // m
    for k in range(levels):
        nb = n // m ** k
        y = x[: nb * m ** k].reshape(nb, m ** k, 3).mean(axis=1)
        assert nins[k] == nb
        for j in range(0 if k == 0 else dmin, p):
            if j >= nb:
                continue
            brute = np.sum(y[j:] * y[: nb - j])
            assert acc[k, j] == pytest.approx(brute, rel=1e-9, abs=1e-9), (k, j)


@pytest.mark.parametrize("p,m,levels,n", [(16, 2, 4, 300), (8, 4, 3, 500)])
def test_msd_correlator_matches_bruteforce(oracle_mod, p, m, levels, n):
    """MSD correlator (type 1, eq_ensemble_kernel.cu:181-189,203,218): level k
    holds every m^k-th position (the first of each block, not an average); lag j
    accumulates sum_i |y_k(i) - y_k(i-j)|^2."""
    rng = np.random.default_rng(2)
    x = rng.standard_normal((n, 3)).cumsum(axis=0)
    acc, nins = oracle_mod.corr_series(x, p, m, levels, kind=1)
    dmin = p // m
    for k in range(levels):
        y = x[:: m ** k][: n // m ** k]
        nb = len(y)
        assert nins[k] == nb
        for j in range(0 if k == 0 else dmin, p):
            if j >= nb:
                continue
            brute = np.sum((y[j:] - y[: nb - j]) ** 2)
            assert acc[k, j] == pytest.approx(brute, rel=1e-9, abs=1e-9), (k, j)


def test_msd_mode_is_diffusive(oracle_mod):
    """Centre-of-mass MSD of an equilibrium melt: zero at lag 0, growing with
    the lag, and the first-entanglement positions move (R1 tracking)."""
    o = oracle_mod.Oracle(nk=20, n_chains=64, seed=5, msd=True, sync_dt=1.0, t_end=200.0, corr_p=16, corr_m=2)
    o.init_equilibrium()
    o.run(200.0)
    g, c = o.gt_raw()
    msd = g.ravel()[c.ravel() > 0] / 64.0
    assert msd[0] == 0.0
    lag = msd[1:12]
    assert np.all(np.diff(lag) > 0), lag
    assert np.abs(o.r1()).max() > 0.0


def test_gex_background_oracle_runs(oracle_mod, dsm_mod):
    """The oracle's GEX partner law: lifetimes of the initial entanglements
    follow the background mixture (a broader law than the monodisperse one:
    partners shorter than N_K renew faster), and the run stays finite."""
    tabs = dsm_mod.gex_tables(1.0, 1.0, 1000.0, 100.0, 1.0)
    assert tabs["step"] > 0 and len(tabs["M"]) > 1000 and tabs["prefact"] > 0
    o = oracle_mod.Oracle(nk=40, n_chains=256, seed=3, gex_tables=tabs)
    m = oracle_mod.Oracle(nk=40, n_chains=256, seed=3)
    o.init_equilibrium()
    m.init_equilibrium()
    so, sm = o.get_state(), m.get_state()
    to = np.concatenate([so["tau"][i, : so["Z"][i] - 1] for i in range(256)])
    tm = np.concatenate([sm["tau"][i, : sm["Z"][i] - 1] for i in range(256)])
    assert np.all(np.isfinite(to)) and np.all(to > 0)
    assert not np.array_equal(np.sort(to), np.sort(tm))
    o.run(20.0)
    assert np.all(o.get_state()["stall"] == 0)
