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
