"""Serving loop (dsm_serve_*): requests batched on one GPU give the results of
the same ensembles run alone through dsm_advance."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHEAR = lambda g: (0.0, g, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0)

REQS = [
    dict(nk=25, n_chains=512, eq_type=1, sync_dt=1.0, t_end=200.0, corr_p=16, corr_m=2, seed=3, stream=0),
    dict(nk=40, n_chains=256, kappa=SHEAR(2e-3), sync_dt=10.0, t_end=60.0, seed=4, stream=1),
    dict(nk=60, n_chains=128, eq_type=1, sync_dt=1.0, t_end=150.0, corr_p=16, corr_m=2, seed=5, stream=2),
    dict(nk=30, n_chains=300, kappa=SHEAR(1e-2), sync_dt=5.0, t_end=40.0, seed=6, stream=3),
]


def _alone(dsm, spec):
    e = dsm.Ensemble(**spec)
    e.init_equilibrium()
    if any(spec.get("kappa", (0.0,) * 9)):
        # outputs at min(t_end, k * sync_dt), as the server computes them
        out = []
        k_max = int(np.ceil(spec["t_end"] / spec["sync_dt"] - 1e-9))
        for k in range(1, k_max + 1):
            e.advance(min(spec["t_end"], k * spec["sync_dt"]))
            out.append(e.stress()[0])
        return np.array(out, np.float32)
    e.advance(spec["t_end"])
    return e.gt()


def _check(srv, ids, dsm):
    for rid, spec in zip(ids, REQS):
        st = srv.status(rid)
        assert st["state"] == dsm.api.REQ_DONE, st
        assert st["latency_s"] >= st["queue_s"] >= 0.0
        ref = _alone(dsm, spec)
        if any(spec.get("kappa", (0.0,) * 9)):
            t, s = srv.result_stress(rid)
            assert np.array_equal(t, np.minimum(spec["t_end"], np.arange(1, len(t) + 1) * spec["sync_dt"]))
            assert np.array_equal(s, ref)  # same windows, same bits
        else:
            t, g = srv.result_gt(rid)
            tr, gr = ref
            assert np.array_equal(t, tr)
            # level-0 lags are flushed to FP64 at each window end: windows differ
            assert np.all(np.abs(g - gr) <= 1e-5 * np.abs(gr).max())


@pytest.mark.parametrize("max_active,chunk_s,policy", [(0, 0.002, "fcfs"), (0, 0.002, "equal_pace"),
                                                        (1, -1.0, "fcfs")])
def test_serve_matches_alone(dsm_mod, max_active, chunk_s, policy):
    with dsm_mod.Server(max_active=max_active, chunk_s=chunk_s, policy=policy) as srv:
        ids = [srv.submit(**r) for r in REQS]
        srv.wait_all(600.0)
        _check(srv, ids, dsm_mod)
        st = srv.stats()
        assert st["completed"] == len(REQS) and st["events"] > 0
        if max_active == 1:
            assert st["peak_active"] == 1


def test_serve_budget_admission(dsm_mod):
    """A budget smaller than the four ensembles together queues some of them."""
    budget = 3 << 20
    with dsm_mod.Server(hbm_budget=budget, chunk_s=0.002) as srv:
        ids = [srv.submit(**r) for r in REQS]
        srv.wait_all(600.0)
        _check(srv, ids, dsm_mod)
        st = srv.stats()
        assert 0 < st["peak_bytes"] <= budget and 1 <= st["peak_active"] < len(REQS)
        with pytest.raises(dsm_mod.DSMError):
            srv.submit(nk=200, n_chains=1 << 20)
