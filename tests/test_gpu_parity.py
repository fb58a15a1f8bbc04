"""GPU (sm_103a, through the C ABI) against the oracle: integer state, event
sequence, Q and lifetimes must agree bit for bit under the shared Philox
streams; stress and G(t) within the stated tolerances."""
import numpy as np
import pytest

from helpers import assert_bitexact, gpu_state, pair

pytestmark = pytest.mark.gpu


def test_init_bitexact(dsm_mod, oracle_mod):
    g, o = pair(dsm_mod, oracle_mod, nk=25, n=1024, seed=1)
    g.init_equilibrium()
    o.init_equilibrium()
    assert_bitexact(gpu_state(g), o.get_state(), keys=("Z", "QN", "tau", "S", "T", "step"), what="init")


@pytest.mark.parametrize("lanes", [0, 32])
@pytest.mark.parametrize("nk,n,steps", [(25, 1024, 3000), (200, 128, 4000), (3, 64, 500), (1, 16, 200)])
def test_fixed_steps_bitexact(dsm_mod, oracle_mod, nk, n, steps, lanes):
    """Default schedule (equilibrium: 16 lanes per chain, small slots) and one
    warp per chain give the oracle's states after a fixed event count."""
    g, o = pair(dsm_mod, oracle_mod, nk=nk, n=n, seed=7, lanes=lanes)
    g.init_equilibrium()
    o.init_equilibrium()
    ev = g.advance(1.0e9, step_limit=steps)
    evo = o.run(1.0e9, step_limit=steps)
    assert ev == evo == n * steps
    assert_bitexact(gpu_state(g), o.get_state(), what=f"nk={nk}")


def test_time_windows_bitexact(dsm_mod, oracle_mod):
    """Chains advanced in several windows on the GPU equal one oracle run."""
    g, o = pair(dsm_mod, oracle_mod, nk=25, n=512, seed=3)
    g.init_equilibrium()
    o.init_equilibrium()
    tot = 0
    for t in (5.0, 17.5, 40.0, 100.0):
        tot += g.advance(t)
    assert tot == o.run(100.0)
    assert_bitexact(gpu_state(g), o.get_state(), what="windows")


@pytest.mark.parametrize("beta,cd", [(0.5, 1), (2.0, 1), (1.0, 0)])
def test_beta_cd_variants_bitexact(dsm_mod, oracle_mod, beta, cd):
    g, o = pair(dsm_mod, oracle_mod, nk=40, n=256, seed=11, beta=beta, cd=cd)
    g.init_equilibrium()
    o.init_equilibrium()
    g.advance(60.0)
    o.run(60.0)
    assert_bitexact(gpu_state(g), o.get_state(), what=f"beta={beta} cd={cd}")


def test_capacity_refusal_bitexact(dsm_mod, oracle_mod):
    """Creation refused at Z == z_max (null events, ensemble_kernel.cu:380,423,451)."""
    g, o = pair(dsm_mod, oracle_mod, nk=30, n=256, seed=5, z_max=14)
    g.init_equilibrium()
    o.init_equilibrium()
    g.advance(1.0e9, step_limit=3000)
    o.run(1.0e9, step_limit=3000)
    st = gpu_state(g)
    assert st["Z"].max() == 14
    assert_bitexact(st, o.get_state(), what="z_max=14")


def test_flow_bitexact(dsm_mod, oracle_mod):
    kap = (0.0, 2.0e-3, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0)
    g, o = pair(dsm_mod, oracle_mod, nk=50, n=256, seed=2, kappa=kap)
    g.init_equilibrium()
    o.init_equilibrium()
    for t in (10.0, 20.0, 30.0):
        g.advance(t)
        o.run(t)
        assert_bitexact(gpu_state(g), o.get_state(), keys=("Z", "QN", "tau", "T", "step", "hash", "S", "stall", "dt_prev"),
                        what=f"flow t={t}")
        sg, cg = g.stress()
        so, co = o.stress()
        assert cg == co
        # per-chain FP32 sums vs FP64: 1e-4 relative to the stress scale
        scale = np.abs(so[:6]).max() + 1e-6
        assert np.all(np.abs(sg[:6] - so[:6]) <= 1e-4 * scale + 1e-6), (sg, so)
        assert abs(sg[6] - so[6]) <= 1e-5 * abs(so[6]) and sg[7] == pytest.approx(so[7], rel=1e-6)


def test_polydisperse_bitexact(dsm_mod, oracle_mod):
    rng = np.random.default_rng(7)
    nkc = rng.integers(10, 120, size=300).astype(np.int32)
    g, o = pair(dsm_mod, oracle_mod, nk=int(nkc.max()), n=300, seed=9, nk_chain=nkc)
    g.init_equilibrium()
    o.init_equilibrium()
    g.advance(30.0)
    o.run(30.0)
    st = gpu_state(g)
    assert np.all(st["QN"][:, :, 3].sum(axis=1) == nkc)
    assert_bitexact(st, o.get_state(), what="polydisperse")


def test_correlator_against_oracle(dsm_mod, oracle_mod):
    """G(t) sums: GPU FP32-compensated level 0 / FP64 long lags vs FP64 oracle."""
    g, o = pair(dsm_mod, oracle_mod, nk=25, n=512, seed=1, corr=True, sync_dt=1.0, t_end=400.0,
                corr_p=16, corr_m=2)
    g.init_equilibrium()
    o.init_equilibrium()
    for t in (100.0, 250.0, 400.0):
        g.advance(t)
    o.run(400.0)
    assert_bitexact(gpu_state(g), o.get_state(), keys=("Z", "QN", "tau", "T", "step", "hash"), what="corr run")
    gs, gc = g.gt_raw()
    os_, oc = o.gt_raw()
    assert np.array_equal(gc, oc)
    mask = oc > 0
    rel = np.abs(gs[mask] - os_[mask]) / np.abs(os_[mask]).max()
    assert rel.max() < 1e-5, rel.max()


def test_set_get_roundtrip(dsm_mod, oracle_mod, tmp_path):
    g, o = pair(dsm_mod, oracle_mod, nk=25, n=64, seed=4)
    g.init_equilibrium()
    g.advance(20.0)
    heads, qn, tau = g.get_chains()
    p = tmp_path / "conf.bin"
    g.save(str(p))
    g2 = dsm_mod.Ensemble(nk=25, n_chains=64, seed=4)
    g2.load(str(p))
    h2, q2, t2 = g2.get_chains()
    assert np.array_equal(heads["Z"], h2["Z"]) and np.array_equal(qn, q2) and np.array_equal(tau, t2)
    # continue both from the loaded conformations: oracle fed the same state
    o.set_state(h2["Z"], q2, t2, T=g2.get_ext()["T"])
    g2.advance(40.0)
    o.run(40.0)
    assert_bitexact(gpu_state(g2), o.get_state(), keys=("Z", "QN", "tau", "T", "step", "hash", "S"),
                    what="loaded")


@pytest.mark.parametrize("kappa", [(0.0,) * 9, (0.0, 1.0e-4, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0)])
def test_long_chains_monodisperse(dsm_mod, oracle_mod, kappa):
    """N_K = 1500: full-capacity slots of 1500 strands do not fit four chains
    per block, so the launch runs fewer warps per block; the chains still give
    the oracle's trajectories exactly, alone and through dsm_advance_batch."""
    g, o = pair(dsm_mod, oracle_mod, nk=1500, n=96, seed=13, kappa=kappa)
    h = dsm_mod.Ensemble(nk=1500, n_chains=96, seed=13, kappa=kappa)
    for x in (g, h, o):
        x.init_equilibrium()
    ev = g.advance(2.0)
    assert ev == o.run(2.0)
    assert dsm_mod.advance_batch([h], 2.0)[0] == ev
    st = o.get_state()
    assert_bitexact(gpu_state(g), st, what="N_K=1500")
    assert_bitexact(gpu_state(h), st, what="N_K=1500 batched")


def test_chain_transfer_layout_and_validation(dsm_mod):
    """dsm_get_chains returns the reference layout (slots beyond Z zero, the
    entanglement slot of the last strand zero), also into caller buffers;
    dsm_set_chains rejects the first bad chain in chain order and accepts the
    state it returned."""
    g = dsm_mod.Ensemble(nk=60, n_chains=9000, seed=5)
    g.init_equilibrium()
    g.advance(30.0)
    heads, qn, tau = g.get_chains()
    Z = heads["Z"].astype(np.int64)
    idx = np.arange(g.z_max)[None, :]
    assert np.all(qn[idx >= Z[:, None]] == 0.0)
    assert np.all(tau[idx >= (Z - 1)[:, None]] == 0.0)
    assert np.all(qn[idx < Z[:, None]][:, 3] >= 1.0)
    out = (np.empty_like(heads), np.full_like(qn, 7.0), np.full_like(tau, 7.0))
    g.get_chains(out=out)
    assert np.array_equal(out[0], heads) and np.array_equal(out[1], qn) and np.array_equal(out[2], tau)
    ok = gpu_state(g)
    bad_q = qn.copy()
    bad_q[8000, 0, 3] += 0.5          # fractional N, later in chain order
    bad_q[6500, 0, 3] += 1.0          # sum of N off by one: the first bad chain
    with pytest.raises(dsm_mod.api.DSMError, match="chain 6500: sum of N"):
        g.set_chains(heads, bad_q, tau)
    bad_h = heads.copy()
    bad_h["Z"][100] = 0
    with pytest.raises(dsm_mod.api.DSMError, match="chain 100: Z out of"):
        g.set_chains(bad_h, qn, tau)
    g.set_chains(heads, qn, tau)
    h2, q2, t2 = g.get_chains()
    assert np.array_equal(q2, qn) and np.array_equal(t2, tau) and np.array_equal(h2["Z"], heads["Z"])
    assert np.array_equal(gpu_state(g)["Z"], ok["Z"])


@pytest.mark.parametrize("kind", ["gt", "flow", "msd"])
def test_checkpoint_exact_resume(dsm_mod, tmp_path, kind):
    """A full-state checkpoint restored into a fresh ensemble continues with
    the same bits as the ensemble that wrote it: chain state, event hash,
    G(t) / MSD sums or stress."""
    kw = dict(nk=60, n_chains=700, seed=19, sync_dt=1.0, t_end=1.0e4)
    if kind == "gt":
        kw.update(eq_type=1, corr_p=16, corr_m=2)
    elif kind == "msd":
        kw.update(eq_type=2, corr_p=16, corr_m=4)
    else:
        kw.update(kappa=(0.0, 2.0e-3, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0))
    a = dsm_mod.Ensemble(**kw)
    a.init_equilibrium()
    a.advance(30.0)
    path = tmp_path / "state.ckpt"
    a.checkpoint(str(path))
    b = dsm_mod.Ensemble(**kw)
    b.restore(str(path))
    for t in (45.0, 70.0):
        ea, eb = a.advance(t), b.advance(t)
        assert ea == eb
        if kind == "flow":
            assert np.array_equal(a.stress()[0], b.stress()[0])
    assert_bitexact(gpu_state(b), gpu_state(a), what=f"restored {kind}")
    if kind != "flow":
        ga, gb = a.gt_raw(), b.gt_raw()
        assert np.array_equal(ga[0], gb[0]) and np.array_equal(ga[1], gb[1])


def test_checkpoint_rejects_mismatch(dsm_mod, tmp_path):
    """Restoring checks the ensemble's shape, random streams and the payload
    checksum first; a rejected restore leaves the ensemble unchanged."""
    kw = dict(nk=40, n_chains=300, seed=23, eq_type=1, sync_dt=1.0, t_end=1.0e4, corr_p=16, corr_m=2)
    a = dsm_mod.Ensemble(**kw)
    a.init_equilibrium()
    a.advance(10.0)
    path = tmp_path / "a.ckpt"
    a.checkpoint(str(path))
    before = gpu_state(a)
    for other, why in ((dict(kw, n_chains=301), "number of chains"), (dict(kw, seed=24), "random streams"),
                       (dict(kw, corr_m=4), "correlator"), (dict(kw, eq_type=0), "correlator")):
        x = dsm_mod.Ensemble(**other)
        x.init_equilibrium()
        with pytest.raises(dsm_mod.api.DSMError, match=why):
            x.restore(str(path))
    raw = bytearray(path.read_bytes())
    raw[len(raw) // 2] ^= 0x40
    bad = tmp_path / "bad.ckpt"
    bad.write_bytes(bytes(raw))
    with pytest.raises(dsm_mod.api.DSMError, match="checksum"):
        a.restore(str(bad))
    (tmp_path / "short.ckpt").write_bytes(bytes(raw[: len(raw) // 3]))
    with pytest.raises(dsm_mod.api.DSMError, match="truncated"):
        a.restore(str(tmp_path / "short.ckpt"))
    assert_bitexact(gpu_state(a), before, what="unchanged after rejected restores")


@pytest.mark.parametrize("nk,n,kappa,z_max", [(25, 1024, (0.0,) * 9, 0), (200, 256, (0.0,) * 9, 0),
                                              (50, 256, (0.0, 2.0e-3, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0), 0),
                                              (30, 256, (0.0,) * 9, 14)])
def test_two_chains_per_warp_bitexact(dsm_mod, oracle_mod, nk, n, kappa, z_max):
    """16 lanes per chain (two chains per warp) reproduce the oracle exactly."""
    g, o = pair(dsm_mod, oracle_mod, nk=nk, n=n, seed=13, kappa=kappa, z_max=z_max, lanes=16)
    g.init_equilibrium()
    o.init_equilibrium()
    for t in (15.0, 40.0):
        g.advance(t)
        o.run(t)
    assert_bitexact(gpu_state(g), o.get_state(), what=f"lanes=16 nk={nk}")


def test_two_chains_per_warp_correlator(dsm_mod, oracle_mod):
    g, o = pair(dsm_mod, oracle_mod, nk=25, n=512, seed=1, corr=True, sync_dt=1.0, t_end=300.0,
                corr_p=16, corr_m=2, lanes=16)
    g.init_equilibrium()
    o.init_equilibrium()
    g.advance(120.0)
    g.advance(300.0)
    o.run(300.0)
    assert_bitexact(gpu_state(g), o.get_state(), keys=("Z", "QN", "tau", "T", "step", "hash"), what="corr lanes=16")
    gs, gc = g.gt_raw()
    os_, oc = o.gt_raw()
    assert np.array_equal(gc, oc)
    mask = oc > 0
    assert (np.abs(gs[mask] - os_[mask]) / np.abs(os_[mask]).max()).max() < 1e-5


def _lognormal_nk(n, seed, mean, sd, lo, hi):
    rng = np.random.default_rng(seed)
    return np.clip(np.round(np.exp(rng.normal(np.log(mean), sd, size=n))), lo, hi).astype(np.int32)


@pytest.mark.parametrize("small_slot,margin,kappa,lanes", [
    (0, 0.0, (0.0,) * 9, 0),
    (40, 0.01, (0.0,) * 9, 0),
    (40, 0.01, (0.0, 1.0e-3, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0), 0),
    (40, 0.01, (0.0,) * 9, 16),
    (40, 0.01, (0.0, 1.0e-3, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0), 16),
])
def test_size_classes_bitexact(dsm_mod, oracle_mod, small_slot, margin, kappa, lanes):
    """Polydisperse chains up to N_K=1200 in size classes (large slots, small
    slots, with two chains per warp also a middle class of one chain per warp,
    overflow launch for chains that outgrow theirs) give the oracle's
    trajectories exactly, whatever the schedule."""
    nkc = _lognormal_nk(400, 21, 120, 0.9, 10, 1200)
    g, o = pair(dsm_mod, oracle_mod, nk=int(nkc.max()), n=400, seed=17, nk_chain=nkc, kappa=kappa)
    if small_slot:
        g.set_schedule(small_slot=small_slot, z_margin_sd=margin, lanes=lanes)
    sch = g.schedule()
    classes, overflow = sch[:-1], sch[-1]
    assert overflow["warps_per_block"] == 1 and overflow["chains"] == 0
    assert sum(k["chains"] for k in classes) == 400 and min(k["chains"] for k in classes) > 0
    assert classes[-1]["warps_per_block"] == 4 and classes[-1]["lanes"] == (16 if lanes == 16 else 32)
    assert classes[0]["warps_per_block"] == 1  # the longest chains: one warp per block
    if lanes == 16:  # a middle class of one chain per warp
        assert any(k["warps_per_block"] == 4 and k["lanes"] == 32 for k in classes)
    g.init_equilibrium()
    o.init_equilibrium()
    deferred = 0
    for t in (4.0, 10.0):
        g.advance(t)
        o.run(t)
        deferred += g.window_stats()["deferred"]
    st = gpu_state(g)
    assert np.all(st["QN"][:, :, 3].sum(axis=1) == nkc)
    assert_bitexact(st, o.get_state(), what=f"size classes slot={small_slot}")
    if small_slot:
        assert deferred > 0  # the overflow launch ran
    if any(kappa):
        sg, cg = g.stress()
        so, co = o.stress()
        assert cg == co
        scale = np.abs(so[:6]).max() + 1e-6
        assert np.all(np.abs(sg[:6] - so[:6]) <= 1e-4 * scale + 1e-6)


@pytest.mark.parametrize("corr", [False, True])
def test_carved_classes_bitexact(dsm_mod, oracle_mod, corr):
    """The carved one-launch form (dsm_set_class_form(1)): large, middle and
    small classes in one launch whose blocks carve their shared memory per
    class, the longest chains beside it, the overflow launch after it.  Same
    trajectories as the oracle (and so as the concurrent launches), with and
    without the G(t) correlator."""
    nkc = _lognormal_nk(400, 21, 120, 0.9, 10, 1200)
    kw = dict(sync_dt=1.0, t_end=1.0e4, corr_p=16, corr_m=2) if corr else {}
    g, o = pair(dsm_mod, oracle_mod, nk=int(nkc.max()), n=400, seed=17, nk_chain=nkc, corr=corr, **kw)
    g.set_schedule(small_slot=40, z_margin_sd=0.01, lanes=16)
    assert g.class_form() == 0
    g.set_class_form(1)
    assert g.class_form() == 1
    sch = g.schedule()
    assert sum(k["chains"] for k in sch[:-1]) == 400
    g.init_equilibrium()
    o.init_equilibrium()
    deferred = 0
    for t in (4.0, 10.0):
        g.advance(t)
        o.run(t)
        deferred += g.window_stats()["deferred"]
    assert deferred > 0  # chains outgrew their carved slot and finished in the overflow launch
    st = gpu_state(g)
    assert np.all(st["QN"][:, :, 3].sum(axis=1) == nkc)
    assert_bitexact(st, o.get_state(), what="carved classes")
    if corr:
        gs, gc = g.gt_raw()
        os_, oc = o.gt_raw()
        assert np.array_equal(gc, oc)
        m = oc > 0
        assert np.max(np.abs(gs[m] - os_[m])) <= 1e-5 * np.abs(os_[m]).max()
    g.set_class_form(0)
    assert g.class_form() == 0


def test_autotune_keeps_trajectory(dsm_mod, oracle_mod):
    """The autotuner's trial windows are ordinary windows under different
    schedules: the run stays on the oracle's trajectory."""
    nkc = _lognormal_nk(300, 5, 150, 0.64, 10, 900)
    g, o = pair(dsm_mod, oracle_mod, nk=int(nkc.max()), n=300, seed=23, nk_chain=nkc, corr=True, sync_dt=1.0,
                t_end=20.0, corr_p=16, corr_m=2)
    g.init_equilibrium()
    o.init_equilibrium()
    g.advance(3.0)
    best = g.autotune(0.5)
    assert best["lanes"] in (16, 32) and best["candidates"] >= 2 and best["kernel_ms"] > 0
    assert g.get_ext()["T"].min() >= (3.0 + 0.5 * best["candidates"]) * 2.0 ** 32 - 1
    g.advance(15.0)
    o.run(15.0)
    assert_bitexact(gpu_state(g), o.get_state(), keys=("Z", "QN", "tau", "T", "step", "hash"), what="after autotune")
    gs, gc = g.gt_raw()
    os_, oc = o.gt_raw()
    assert np.array_equal(gc, oc)
    mask = oc > 0
    assert (np.abs(gs[mask] - os_[mask]) / np.abs(os_[mask]).max()).max() < 1e-5


def test_graph_series_equals_windows(dsm_mod, oracle_mod):
    """n windows replayed from one captured CUDA graph equal n dsm_advance
    calls (state bit for bit, stress after every window) and the oracle."""
    kap = (0.0, 3.0e-3, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0)
    spec = dict(nk=40, n_chains=300, kappa=kap, seed=29)
    a = dsm_mod.Ensemble(**spec)
    b = dsm_mod.Ensemble(**spec)
    o = oracle_mod.Oracle(**spec)
    for x in (a, b, o):
        x.init_equilibrium()
    sa = []
    for w in range(1, 6):
        a.advance(2.5 * w)
        sa.append(a.stress()[0])
    ev1, sb = b.advance_series(2.5, 5)
    assert np.array_equal(np.array(sa, np.float32), sb)
    assert_bitexact(gpu_state(b), gpu_state(a), what="series vs windows")
    o.run(12.5)
    assert_bitexact(gpu_state(b), o.get_state(), what="series vs oracle")
    # replay of the same graph for the next 5 windows
    for w in range(6, 11):
        a.advance(2.5 * w)
    ev2, sb2 = b.advance_series(2.5, 5)
    assert ev2 > 0 and np.array_equal(sb2[-1], a.stress()[0].astype(np.float32))
    assert_bitexact(gpu_state(b), gpu_state(a), what="series replay")


def test_series_size_classes(dsm_mod, oracle_mod):
    """An equilibrium series of a melt in size classes (its windows issued
    directly on the handle's streams, not from a graph), twice in a row:
    events and state equal the oracle's."""
    nkc = _lognormal_nk(300, 31, 150, 0.64, 10, 900)
    g, o = pair(dsm_mod, oracle_mod, nk=int(nkc.max()), n=300, seed=37, nk_chain=nkc)
    g.set_schedule(small_slot=48, z_margin_sd=0.01)
    g.init_equilibrium()
    o.init_equilibrium()
    ev, _ = g.advance_series(1.5, 4)
    assert ev == o.run(6.0)
    assert_bitexact(gpu_state(g), o.get_state(), what="series with size classes")
    ev, _ = g.advance_series(1.5, 3)
    assert ev == o.run(10.5)
    assert g.window_stats()["events"] == ev
    assert_bitexact(gpu_state(g), o.get_state(), what="second series with size classes")


@pytest.mark.parametrize("lanes", [0, 32])
def test_flow_series_groups(dsm_mod, oracle_mod, lanes):
    """A flow series runs up to 16 output windows inside one step launch
    (stress recorded at every window end): 40 short windows (about three
    events per chain each, so some chains cross windows without an event)
    equal 40 dsm_advance calls, stress after every window and state bit for
    bit, with one chain stalled (NaN conformation) left out of every sum; the
    state also equals the oracle's."""
    kap = (0.0, 4.0e-3, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0)
    spec = dict(nk=40, n_chains=300, kappa=kap, seed=41, lanes_per_chain=lanes)
    a = dsm_mod.Ensemble(**spec)
    b = dsm_mod.Ensemble(**spec)
    o = oracle_mod.Oracle(nk=40, n_chains=300, kappa=kap, seed=41)
    for x in (a, b, o):
        x.init_equilibrium()
    ev_o = o.run(1.0)
    for x in (a, b):
        assert x.advance(1.0) == ev_o
    assert_bitexact(gpu_state(a), o.get_state(), what="start")
    dt, n = 0.3, 40
    sa, ev_a = [], 0
    for w in range(1, n + 1):
        ev_a += a.advance(1.0 + dt * w)
        sa.append(a.stress()[0])
    ev_b, sb = b.advance_series(dt, n)
    assert ev_b == ev_a
    assert np.array_equal(np.array(sa, np.float32), sb)
    assert_bitexact(gpu_state(b), gpu_state(a), what="flow series vs windows")
    assert ev_a == o.run(1.0 + dt * n)
    assert_bitexact(gpu_state(b), o.get_state(), what="flow series vs oracle")
    # one chain stalls at its next event; it stays out of every window's sum
    for x in (a, b):
        heads, qn, tau = x.get_chains()
        qn[7, 1, 0] = np.nan
        x.set_chains(heads, qn, tau)
    t0, sa = 1.0 + dt * n, []
    for w in range(1, 21):
        a.advance(t0 + dt * w)
        sa.append(a.stress())
    _, sb = b.advance_series(dt, 20)
    assert all(c == 299 for _, c in sa)
    assert np.array_equal(np.array([s for s, _ in sa], np.float32), sb)
    assert_bitexact(gpu_state(b), gpu_state(a), what="flow series with a stalled chain")


def test_flow_series_size_classes(dsm_mod, oracle_mod):
    """Flow series of a polydisperse melt in size classes: a chain that
    outgrows its small slot inside a window group finishes the remaining
    windows of the group in the overflow launch, with the same stress and
    state as separate windows and the oracle."""
    nkc = _lognormal_nk(300, 43, 120, 0.6, 10, 700)
    kap = (0.0, 2.0e-3, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0)
    g, o = pair(dsm_mod, oracle_mod, nk=int(nkc.max()), n=300, seed=47, nk_chain=nkc, kappa=kap)
    h = dsm_mod.Ensemble(nk=int(nkc.max()), n_chains=300, seed=47, nk_chain=nkc, kappa=kap)
    for x in (g, h):
        x.set_schedule(small_slot=40, z_margin_sd=0.01)
        x.init_equilibrium()
    o.init_equilibrium()
    sh, ev_h = [], 0
    for w in range(1, 25):
        ev_h += h.advance(0.5 * w)
        sh.append(h.stress()[0])
    ev, sg = g.advance_series(0.5, 24)
    assert ev == ev_h == o.run(12.0)
    assert np.array_equal(np.array(sh, np.float32), sg)
    assert_bitexact(gpu_state(g), gpu_state(h), what="flow series in size classes vs windows")
    assert_bitexact(gpu_state(g), o.get_state(), what="flow series in size classes vs oracle")
    assert g.window_stats()["deferred"] > 0


@pytest.mark.parametrize("lanes", [0, 32])
def test_msd_mode(dsm_mod, oracle_mod, lanes):
    """MSD mode (eq_type=2): chain state and the first-entanglement positions
    R1 bit for bit, MSD(t) sums within 1e-4 of the FP64 oracle (FP32 centre of
    mass from tile scans on the GPU)."""
    g, o = pair(dsm_mod, oracle_mod, nk=30, n=512, seed=8, msd=True, sync_dt=1.0, t_end=300.0, corr_p=16, corr_m=2,
                lanes=lanes)
    g.init_equilibrium()
    o.init_equilibrium()
    for t in (70.0, 300.0):
        g.advance(t)
    o.run(300.0)
    assert_bitexact(gpu_state(g), o.get_state(), keys=("Z", "QN", "tau", "T", "step", "hash"), what="msd")
    r1g, r1o = g.r1(), o.r1()
    assert np.array_equal(r1g, r1o.astype(np.float32)) and np.abs(r1o).max() > 0
    gs, gc = g.gt_raw()
    os_, oc = o.gt_raw()
    assert np.array_equal(gc, oc)
    mask = oc > 0
    assert (np.abs(gs[mask] - os_[mask]) / np.abs(os_[mask]).max()).max() < 1e-4
    t, msd = g.gt()
    assert msd[0] == 0.0 and np.all(np.diff(msd[1:12]) > 0)


def test_device_distributions(dsm_mod):
    """-distr statistics computed on the device equal the host computation from
    the downloaded conformations (ensemble.cu:356-484)."""
    nkc = _lognormal_nk(500, 3, 60, 0.5, 10, 300)
    g = dsm_mod.Ensemble(nk=int(nkc.max()), n_chains=500, seed=3, nk_chain=nkc)
    g.init_equilibrium()
    g.advance(20.0)
    hz, hn, q = g.distributions()
    heads, qn, _ = g.get_chains()
    Z = heads["Z"]
    assert np.array_equal(hz, np.bincount(Z, minlength=len(hz)).astype(np.uint64))
    ns = np.concatenate([qn[i, :Z[i], 3] for i in range(len(Z))]).astype(np.int64)
    assert np.array_equal(hn, np.bincount(ns, minlength=len(hn)).astype(np.uint64))
    inner = np.concatenate([qn[i, 1:Z[i] - 1, :3] for i in range(len(Z)) if Z[i] > 2])
    ql = np.sort(np.sqrt((inner.astype(np.float64) ** 2).sum(axis=1)))
    assert len(q) == len(ql) and np.all(np.diff(q) >= 0)
    assert np.allclose(q, ql, rtol=1e-6, atol=1e-7)


@pytest.mark.parametrize("beta,kappa", [(1.0, (0.0,) * 9), (2.0, (0.0,) * 9),
                                        (1.0, (0.0, 2.0e-3, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0))])
def test_gex_background_bitexact(dsm_mod, oracle_mod, beta, kappa):
    """GEX background polydispersity (pd_flag = 1, polydisp.dat a b mp Mk):
    partner masses from the inverse tables, p_cd evaluated per new
    entanglement on the device; bit for bit against the oracle fed the same
    tables."""
    gex = (1.0, 1.0, 1000.0, 100.0)
    tabs = dsm_mod.gex_tables(*gex, beta)
    g = dsm_mod.Ensemble(nk=40, n_chains=384, beta=beta, kappa=kappa, seed=19, gex=gex)
    o = oracle_mod.Oracle(nk=40, n_chains=384, beta=beta, kappa=kappa, seed=19, gex_tables=tabs)
    g.init_equilibrium()
    o.init_equilibrium()
    for t in (10.0, 30.0):
        g.advance(t)
        o.run(t)
    assert_bitexact(gpu_state(g), o.get_state(), what=f"gex beta={beta}")


def test_chain_offset_shards_equal_one_ensemble(dsm_mod):
    """Two handles holding chains [0, n/2) and [n/2, n) of one ensemble
    (chain_offset) reproduce the single handle's chains bit for bit: random
    streams are keyed by global chain id, so sharding over GPUs changes
    nothing."""
    n = 512
    spec = dict(nk=40, seed=31, eq_type=1, sync_dt=1.0, t_end=50.0, corr_p=16, corr_m=2)
    whole = dsm_mod.Ensemble(n_chains=n, **spec)
    parts = [dsm_mod.Ensemble(n_chains=n // 2, chain_offset=k * (n // 2), **spec) for k in range(2)]
    for e in [whole] + parts:
        e.init_equilibrium()
        e.advance(50.0)
    sw = gpu_state(whole)
    for k, e in enumerate(parts):
        sp = gpu_state(e)
        sl = slice(k * n // 2, (k + 1) * n // 2)
        assert_bitexact(sp, {key: sw[key][sl] for key in sw}, keys=("Z", "QN", "tau", "T", "step", "hash"),
                        what=f"shard {k}")
    gw, _ = whole.gt_raw()
    gp = sum(e.gt_raw()[0] for e in parts)
    assert np.allclose(gp, gw, rtol=1e-12, atol=0.0)


def test_resident_blocks_by_kind(dsm_mod, oracle_mod):
    """The build for 6 blocks per SM is taken when the slots leave the shared
    memory for it: without a correlator as soon as more blocks fit (N_K = 100,
    16 lanes: 33 KB blocks), with G(t) only at half as many blocks again
    (N_K = 25, p = 16: 6 blocks).  The default schedule picks a smaller slot
    that keeps 6 blocks when the chains fit it (N_K = 100 with G(t), p = 64),
    and keeps 4 blocks when they do not (N_K = 200, p = 64).  The 6-block runs
    equal the oracle."""
    kap = (0.0, 2.0e-3, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0)
    cases = [(100, dict(kappa=kap), 6), (100, dict(), 6), (100, dict(corr=True, t_end=400.0, corr_p=64, corr_m=8), 6),
             (25, dict(corr=True, t_end=400.0, corr_p=16, corr_m=2), 6),
             (200, dict(corr=True, t_end=400.0, corr_p=64, corr_m=8), 4)]
    for nk, kw, bps in cases:
        g, o = pair(dsm_mod, oracle_mod, nk=nk, n=2048, seed=53, **kw)
        g.init_equilibrium()
        o.init_equilibrium()
        ev = g.advance(2.0)
        assert g.last_window()["blocks_per_sm"] == bps, kw
        if bps == 6:
            assert ev == o.run(2.0)
            assert_bitexact(gpu_state(g), o.get_state(), what=f"6-block build {kw}")


def test_observables_independent_of_tile_width(dsm_mod):
    """Stress sums over the strands of a chain take the same order for 16- and
    32-lane tiles, so the flow stress and the G(t) sums do not depend on where
    a chain ran: one chain per warp and two per warp give the same bits."""
    kap = (0.0, 3.0e-3, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0)
    specs = [dict(nk=70, n_chains=400, kappa=kap, seed=61),
             dict(nk=70, n_chains=400, eq_type=1, sync_dt=1.0, t_end=200.0, corr_p=16, corr_m=2, seed=62)]
    for spec in specs:
        a = dsm_mod.Ensemble(**spec, lanes_per_chain=16)
        b = dsm_mod.Ensemble(**spec, lanes_per_chain=32)
        for x in (a, b):
            x.init_equilibrium()
            x.advance(40.0)
        assert_bitexact(gpu_state(a), gpu_state(b), what="16 vs 32 lanes")
        if "kappa" in spec:
            assert np.array_equal(a.stress()[0], b.stress()[0])
        else:
            ga, ca = a.gt_raw()
            gb, cb = b.gt_raw()
            assert np.array_equal(ca, cb) and np.array_equal(ga, gb)


def test_equilibrium_stress_against_oracle(dsm_mod, oracle_mod):
    """dsm_stress of an equilibrium ensemble (evaluated from the current state,
    as calc_stress does for any ensemble, ensemble.cu:210-221) against the
    oracle's FP64 average of the same chains."""
    g, o = pair(dsm_mod, oracle_mod, nk=40, n=512, seed=13, corr=True, sync_dt=1.0, t_end=60.0)
    g.init_equilibrium()
    o.init_equilibrium()
    g.advance(60.0)
    o.run(60.0)
    assert_bitexact(gpu_state(g), o.get_state(), keys=("Z", "QN", "tau", "T", "step", "hash"), what="eq stress run")
    sg, cg = g.stress()
    so, co = o.stress()
    assert cg == co == 512
    scale = np.abs(so[:6]).max() + 1e-6
    assert np.all(np.abs(sg[:6] - so[:6]) <= 1e-5 * scale), (sg, so)
    assert sg[6] == pytest.approx(so[6], rel=1e-5) and sg[7] == pytest.approx(so[7], rel=1e-6)
