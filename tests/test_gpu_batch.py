"""Several ensembles in one persistent launch (dsm_advance_batch) give exactly
the states of separate dsm_advance calls and of the oracle."""
import numpy as np
import pytest

from helpers import assert_bitexact, gpu_state

pytestmark = pytest.mark.gpu


def test_batch_equals_separate(dsm_mod, oracle_mod):
    shear = lambda g: (0.0, g, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0)
    specs = [dict(nk=40, n_chains=300, kappa=shear(1e-3), seed=2, stream=0),
             dict(nk=60, n_chains=200, kappa=shear(5e-3), seed=2, stream=1),
             dict(nk=30, n_chains=500, seed=5, stream=2),
             dict(nk=50, n_chains=100, seed=6, stream=3, eq_type=1, sync_dt=1.0, t_end=80.0, corr_p=16, corr_m=2)]
    batch = [dsm_mod.Ensemble(**s) for s in specs]
    single = [dsm_mod.Ensemble(**s) for s in specs]
    for e in batch + single:
        e.init_equilibrium()
    for t in (25.0, 80.0):
        ev_b = dsm_mod.advance_batch(batch, [t, t * 0.5, t, t])
        ev_s = [e.advance(tt) for e, tt in zip(single, [t, t * 0.5, t, t])]
        assert list(ev_b) == ev_s
        for b, s in zip(batch, single):
            assert_bitexact(gpu_state(b), gpu_state(s), what="batch vs single")
        for k in (0, 1):
            sb, cb = batch[k].stress()
            ss, cs = single[k].stress()
            assert cb == cs and np.array_equal(sb, ss)
    gb, cb = batch[3].gt_raw()
    gs, cs = single[3].gt_raw()
    assert np.array_equal(cb, cs) and np.array_equal(gb, gs)
    # and one of them against the oracle
    o = oracle_mod.Oracle(nk=60, n_chains=200, kappa=shear(5e-3), seed=2, stream=1)
    o.init_equilibrium()
    o.run(12.5)
    o.run(40.0)
    assert_bitexact(gpu_state(batch[1]), o.get_state(), what="batch vs oracle")


def test_batch_small_slots_overflow(dsm_mod, oracle_mod):
    """Ensembles whose own schedules run small slots are batched in the
    smallest of them; chains that outgrow it finish in the batch's overflow
    launch.  Shear and equilibrium ensembles, slots forced small so that many
    chains are handed over: events and state equal separate dsm_advance calls
    and the oracle."""
    shear = lambda g: (0.0, g, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0)
    specs = [dict(nk=60, n_chains=300, kappa=shear(2e-3), seed=12, stream=0),
             dict(nk=60, n_chains=200, kappa=shear(8e-3), seed=12, stream=1),
             dict(nk=50, n_chains=256, seed=13, stream=2),
             dict(nk=70, n_chains=128, seed=14, stream=3)]
    batch = [dsm_mod.Ensemble(**s) for s in specs]
    single = [dsm_mod.Ensemble(**s) for s in specs]
    for e, slot in zip(batch + single, [30, 28, 26, 34] * 2):
        e.set_schedule(small_slot=slot, z_margin_sd=0.01)
        e.init_equilibrium()
    deferred = 0
    for t in (6.0, 15.0):
        ev_b = dsm_mod.advance_batch(batch, t)
        deferred += sum(e.window_stats()["deferred"] for e in batch)
        ev_s = [e.advance(t) for e in single]
        assert list(ev_b) == ev_s
        for b, s in zip(batch, single):
            assert_bitexact(gpu_state(b), gpu_state(s), what="batch with overflow vs single")
        for k in (0, 1):
            assert np.array_equal(batch[k].stress()[0], single[k].stress()[0])
    assert deferred > 0
    o = oracle_mod.Oracle(nk=60, n_chains=200, kappa=shear(8e-3), seed=12, stream=1)
    o.init_equilibrium()
    o.run(15.0)
    assert_bitexact(gpu_state(batch[1]), o.get_state(), what="batch with overflow vs oracle")


def test_async_handles_overlap(dsm_mod, oracle_mod):
    """Windows and graph series enqueued on several handles at once (each on
    its own stream) and polled give the synchronous results."""
    import time

    kap = (0.0, 2.0e-3, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0)
    specs = [dict(nk=30, n_chains=400, seed=3), dict(nk=45, n_chains=300, kappa=kap, seed=3, stream=1)]
    a = [dsm_mod.Ensemble(**s) for s in specs]
    b = [dsm_mod.Ensemble(**s) for s in specs]
    for e in a + b:
        e.init_equilibrium()
    a[0].advance_start(20.0)
    a[1].series_start([4.0, 8.0, 12.0])
    res = [None, None]
    t0 = time.time()
    while any(r is None for r in res) and time.time() - t0 < 60:
        for i in range(2):
            if res[i] is None:
                res[i] = a[i].poll()
    ev0 = b[0].advance(20.0)
    st1 = []
    ev1 = 0
    for t in (4.0, 8.0, 12.0):
        ev1 += b[1].advance(t)
        st1.append(b[1].stress()[0])
    assert res[0][0] == ev0 and res[1][0] == ev1
    assert np.array_equal(res[1][1], np.array(st1, np.float32))
    for x, y in zip(a, b):
        assert_bitexact(gpu_state(x), gpu_state(y), what="async vs sync")
