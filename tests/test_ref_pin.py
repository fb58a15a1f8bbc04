"""The oracle pinned against the reference's own kMC kernels.

oracle/ref_step.cpp compiles strent_kernel, chain_kernel, stress_calc
(common/ensemble_kernel.cu) and EQ_strent_kernel, EQ_chain_kernel, corr_add,
update_correlator (common/eq_ensemble_kernel.cu) unchanged for the host and
drives them with the step loops of common/ensemble_call_block.cu (ping-pong
arrays, delayed dynamics, sync windows, 250-step rings).  Fed the random
stream of oracle/ref_tape.h, the reference kernels and the oracle's
reference-arithmetic mode (mode 2) must give the same chains bit for bit
(Z, N, Q, lifetimes, FP32 clocks, sample counters, R1) and the same G(t), MSD
and flow stress up to the FP32 sums of the reference.

Then the chain of evidence to the GPU: the sm_103a kernel reproduces mode 0
bit for bit (test_gpu_parity.py); mode 0 and mode 2 share their random words,
so the two arithmetics follow the identical event sequence until a rounding
difference flips one decision, which happens on about one event in 10^6.

Where the reference tree is absent, mode 2 is checked against
tests/golden/ref_step_reference.npz, written from the compiled reference
kernels by tests/golden/make_golden.py."""
from pathlib import Path

import numpy as np
import pytest

GOLD = Path(__file__).resolve().parent / "golden" / "ref_step_reference.npz"
XY = (0.0, 2.0e-3, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0)


@pytest.fixture(scope="module")
def refstep(oracle_mod):
    if oracle_mod.refstep_lib() is None:
        pytest.skip("reference tree not available (the golden-fixture test covers this case)")
    return oracle_mod


def _pair(orc, *, nk, n, seed=3, kappa=(0.0,) * 9, cd=1, beta=1.0, z_max=0, corr=True, msd=False, t_end=1000.0,
          p=16, m=2, init="oracle"):
    flow = any(k != 0 for k in kappa)
    o = orc.Oracle(nk=nk, n_chains=n, mode=2, seed=seed, kappa=kappa, cd_flag=cd, beta=beta, z_max=z_max,
                   corr=corr and not flow, msd=msd, sync_dt=1.0, t_end=t_end, corr_p=p, corr_m=m)
    if init == "reference":
        # chains from the reference's own initialiser (chain.cu:199-283, MT19937 seeded job_ID * N_cha)
        import ctypes as C
        R = orc.ref_lib()
        zc = o.cap
        Z = np.zeros(n, np.int32)
        QN = np.zeros((n, zc, 4), np.float32)
        tau = np.zeros((n, zc), np.float32)
        R.ref_chain_init(seed * n, n, nk, C.c_float(beta), cd, zc, Z.ctypes.data_as(C.c_void_p),
                         QN.ctypes.data_as(C.c_void_p), tau.ctypes.data_as(C.c_void_p))
        o.set_state(Z, QN, tau)
        st = {"Z": Z, "QN": QN, "tau": tau}
    else:
        o.init_equilibrium()
        st = o.get_state()
    r = orc.RefStep(o, corr_res=1)
    r.set_chains(st["Z"], st["QN"], st["tau"])
    return o, r


def _assert_same(o, r, *, cd=1, what=""):
    a, b = o.get_state(), r.get_state()
    tf, k, r1 = o.ref_clock()
    assert np.array_equal(a["Z"], b["Z"]), what
    assert np.array_equal(a["step"].astype(np.int64), b["events"]), what
    assert np.array_equal(a["stall"], b["stall"]), what
    Z = a["Z"]
    idx = np.arange(a["QN"].shape[1])[None, :] < Z[:, None]
    # values compared as floats: the reference's extra zero-dt deformation
    # passes of chains that stopped early may turn -0.0 into +0.0
    assert np.array_equal(a["QN"][idx], b["QN"][idx]), what
    if cd:
        tidx = np.arange(a["tau"].shape[1])[None, :] < (Z - 1)[:, None]
        assert np.array_equal(a["tau"][tidx].view(np.uint32), b["tau"][tidx].view(np.uint32)), what
    assert np.array_equal(tf.view(np.uint32), b["time"].view(np.uint32)), what
    assert np.array_equal(k, b["corr_time"]), what
    assert np.array_equal(r1.view(np.uint32), b["R1"][:, :3].view(np.uint32)), what


CASES = {
    "eq_nk25": dict(nk=25, n=64),
    "eq_nk200": dict(nk=200, n=12),
    "eq_beta0.5": dict(nk=40, n=48, beta=0.5),
    "eq_beta2": dict(nk=40, n=48, beta=2.0),
    "eq_cd_off": dict(nk=40, n=48, cd=0),
    "eq_capacity": dict(nk=30, n=48, z_max=14),
    "eq_nk3": dict(nk=3, n=64),
    "eq_nk2": dict(nk=2, n=64),
    "eq_ref_init": dict(nk=25, n=64, init="reference"),
    "msd": dict(nk=25, n=48, msd=True),
    "flow_nk50": dict(nk=50, n=32, kappa=XY),
    "flow_cd_off": dict(nk=50, n=32, kappa=XY, cd=0),
    "flow_capacity": dict(nk=40, n=32, kappa=XY, z_max=16),
    "flow_strong": dict(nk=25, n=48, kappa=(0.0, 0.5, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0)),
    "flow_extension": dict(nk=25, n=48, kappa=(0.05, 0.0, 0.0, 0.0, -0.025, 0.0, 0.0, 0.0, -0.025)),
}


@pytest.mark.parametrize("case", sorted(CASES))
def test_reference_kernels_fixed_events(refstep, case):
    """After fixed event counts the reference kernels and mode 2 hold the same chains."""
    kw = dict(CASES[case])
    for limit in (1, 7, 300, 2500):
        o, r = _pair(refstep, **kw)
        ev = o.run(9.0e4, limit)
        assert r.run(9.0e4, limit) == 0
        _assert_same(o, r, cd=kw.get("cd", 1), what=f"{case} after {limit} events")
        st = o.get_state()
        assert ev == int(st["step"].sum())
        assert np.all(st["step"][st["stall"] == 0] == limit)  # stalled chains stop early, on both sides


@pytest.mark.parametrize("flow", [False, True])
def test_reference_kernels_time_windows(refstep, flow):
    """Runs to successive times: reach rule, sample rule (equilibrium), window clocks."""
    o, r = _pair(refstep, nk=25, n=64, seed=5, kappa=XY if flow else (0.0,) * 9, t_end=400.0)
    for t in (30.0, 75.0, 160.0, 400.0):
        o.run(t)
        assert r.run(t) == 0
        _assert_same(o, r, what=f"t={t}")


def test_reference_kernels_sync_windows(refstep):
    """A run longer than the reference's 1e5 sync interval (two windows, universal time)."""
    o, r = _pair(refstep, nk=6, n=8, seed=9, t_end=2.2e5)
    o.run(2.2e5)
    assert r.run(2.2e5) == 0
    _assert_same(o, r, what="two sync windows")
    tf, k, _ = o.ref_clock()
    assert np.all(k >= 220000)


def test_reference_correlator(refstep):
    """G(t) ensemble sums: the reference's FP32 corr_add / corr_function_calc_kernel
    vs mode 2's FP64 correlator over the same samples."""
    o, r = _pair(refstep, nk=25, n=64, seed=5, t_end=400.0)
    o.run(400.0)
    assert r.run(400.0) == 0
    _assert_same(o, r, what="G(t) run")
    g, c = o.gt_raw()
    rg, lag, n0 = r.gt()
    assert np.array_equal(c[0], n0[0].astype(np.int64))
    mask = c > 0
    assert np.max(np.abs(g[mask] - rg[mask])) <= 2e-6 * np.abs(g[mask]).max()


def test_reference_msd(refstep):
    """MSD mode (correlator type 1): R1 bit for bit, MSD sums within FP32 rounding."""
    o, r = _pair(refstep, nk=25, n=48, seed=8, msd=True, t_end=300.0)
    o.run(300.0)
    assert r.run(300.0) == 0
    _assert_same(o, r, what="MSD run")
    g, c = o.gt_raw()
    rg, _, _ = r.gt()
    mask = c > 0
    assert np.max(np.abs(g[mask] - rg[mask])) <= 2e-6 * np.abs(g[mask]).max()


def test_reference_flow_stress(refstep):
    """stress_calc + the host average of calc_stress_call_block vs mode 2's FP64 stress."""
    o, r = _pair(refstep, nk=50, n=64, seed=2, kappa=XY)
    for t in (10.0, 20.0, 40.0):
        o.run(t)
        assert r.run(t) == 0
        _assert_same(o, r, what=f"flow t={t}")
        so, co = o.stress()
        sr, cr = r.stress()
        assert co == cr
        assert np.all(np.abs(so[:6] - sr[:6]) <= 2e-6 * np.abs(so[:6]).max())
        assert sr[6] == pytest.approx(so[6], rel=2e-6) and sr[7] == pytest.approx(so[7], rel=1e-7)


def test_reference_fixture(oracle_mod):
    """Mode 2 against reference-kernel outputs committed as a fixture (runs
    without the reference tree)."""
    d = np.load(GOLD)
    for case in [str(c) for c in d["cases"]]:
        g = {k[len(case) + 1:]: d[k] for k in d.files if k.startswith(case + "/")}
        kap = tuple(float(v) for v in g["kappa"])
        o = oracle_mod.Oracle(nk=int(g["nk"]), n_chains=int(g["n"]), mode=2, seed=int(g["seed"]), kappa=kap,
                              corr=not any(kap), sync_dt=1.0, t_end=float(g["t_end"]), corr_p=16, corr_m=2)
        o.set_state(g["Z0"], g["QN0"], g["tau0"])
        o.run(float(g["t_end"]), int(g["limit"]))
        a = o.get_state()
        tf, k, _ = o.ref_clock()
        assert np.array_equal(a["Z"], g["Z"]), case
        Z = a["Z"]
        idx = np.arange(a["QN"].shape[1])[None, :] < Z[:, None]
        assert np.array_equal(a["QN"][idx], g["QN"][idx]), case
        assert np.array_equal(tf.view(np.uint32), g["time"].view(np.uint32)), case
        assert np.array_equal(a["step"].astype(np.int64), g["events"]), case
        if "G" in g:
            gs, c = o.gt_raw()
            mask = c > 0
            assert np.max(np.abs(gs[mask] - g["G"][mask])) <= 2e-6 * np.abs(gs[mask]).max(), case


@pytest.mark.parametrize("nk,n,events,min_same", [(25, 256, 20000, 0.97), (200, 48, 20000, 0.9)])
def test_gpu_arithmetic_follows_reference_arithmetic(oracle_mod, nk, n, events, min_same):
    """Mode 0 (the GPU kernel's arithmetic: fixed-point pick, per-N rate tables,
    own exp/log) and mode 2 (the reference's FP32 rates and running-sum scan)
    draw the same random words; over 2e4 events per chain nearly every chain
    takes the identical event sequence (event hashes equal)."""
    s = {}
    for mode in (0, 2):
        o = oracle_mod.Oracle(nk=nk, n_chains=n, mode=mode, seed=3)
        o.init_equilibrium()
        o.run(9.0e4 if mode == 2 else 1.0e9, events)
        s[mode] = o.get_state()
    same = s[0]["hash"] == s[2]["hash"]
    assert np.all(s[0]["step"] == events) and np.all(s[2]["step"] == events)
    assert same.mean() >= min_same, same.mean()
    # where the sequences agree, so do the chains' integer states
    assert np.array_equal(s[0]["Z"][same], s[2]["Z"][same])
    Z = s[0]["Z"]
    idx = (np.arange(s[0]["QN"].shape[1])[None, :] < Z[:, None]) & same[:, None]
    assert np.array_equal(s[0]["QN"][idx][:, 3], s[2]["QN"][idx][:, 3])
