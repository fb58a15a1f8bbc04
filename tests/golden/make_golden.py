"""Generate the golden fixtures of tests/golden/ from the reference's own host
code (common/chain.cu, common/pcd_tau.h, common/random.h of ktaletsk/gpu_dsm),
compiled from the reference tree by `make -C oracle ref` into
oracle/_ref/libdsmref.so.  Run in a checkout where that tree exists:

    python tests/golden/make_golden.py

Outputs (small JSON files, committed):
  pcd_reference.json    p_cd fit constants (float, pcd_tau.h:32-66) on a grid
  init_reference.json   statistics of reference chain_init ensembles
                        (chain.cu:199-283): Z histogram, N histogram, Q moments,
                        lifetime-rate quantiles
  tau_reference.json    quantiles of the reference lifetime samplers
                        (pcd_tau.h:67-82)
  gex_reference.json    GEX background-MW tables of the reference's
                        make_gamma_table (gamma.cpp:174-263), every 100th entry,
                        from oracle/_ref/ref_gex (a separate process: the
                        reference reads uninitialised memory at the end of the
                        CD-weighted inversion, see oracle/ref_gex_main.cpp)
  ref_step_reference.npz  chains advanced by the reference's own kMC kernels
                        (common/ensemble_kernel.cu, common/eq_ensemble_kernel.cu
                        compiled for the host, oracle/_ref/libdsmrefstep.so) on
                        the random stream of oracle/ref_tape.h: initial and final
                        chains, FP32 clocks, event counts and G(t) sums, for the
                        equilibrium and flow kernels (written on x86_64 glibc,
                        whose expf/powf both sides use)
"""
from __future__ import annotations

import ctypes as C
import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))
from oracle import oracle as orc  # noqa: E402

PCD_NAMES = ["alpha", "tau_0", "tau_max", "tau_d", "g", "c1", "cm1", "rcm1c1", "At", "Adt", "Bdt", "normdt"]
QUANTS = [0.001, 0.01, 0.05, 0.1, 0.2, 0.3, 0.4, 0.5, 0.6, 0.7, 0.8, 0.9, 0.95, 0.99]


def main():
    R = orc.ref_lib()
    if R is None:
        raise SystemExit("reference tree not available: cannot regenerate golden fixtures")
    # ---- p_cd
    rows = []
    for beta in (0.5, 1.0, 2.0, 5.0):
        for nk in (2, 3, 5, 10, 25, 50, 100, 150, 200, 500, 2000):
            out = np.zeros(12, np.float64)
            R.ref_pcd(C.c_float(beta), C.c_float(nk), out.ctypes.data_as(C.c_void_p))
            rows.append({"beta": beta, "nk": nk, **{k: float(v) for k, v in zip(PCD_NAMES, out)}})
    (HERE / "pcd_reference.json").write_text(json.dumps({"source": "common/pcd_tau.h:32-66 (compiled)", "rows": rows}, indent=1))

    # ---- initial ensembles
    ens = []
    for beta, nk, n, seed in ((1.0, 25, 20000, 1), (1.0, 200, 4000, 2), (2.0, 50, 10000, 3), (0.5, 40, 8000, 4)):
        z_max = nk
        Z = np.zeros(n, np.int32)
        QN = np.zeros((n, z_max, 4), np.float32)
        tau = np.zeros((n, z_max), np.float32)
        R.ref_chain_init(seed * n, n, nk, C.c_float(beta), 1, z_max, Z.ctypes.data_as(C.c_void_p),
                         QN.ctypes.data_as(C.c_void_p), tau.ctypes.data_as(C.c_void_p))
        zh = np.bincount(Z, minlength=nk + 1)[: nk + 1]
        Ns, q2n, ends_q = [], [], []
        rates = []
        for i in range(n):
            z = Z[i]
            Ns.extend(QN[i, :z, 3].astype(int).tolist())
            if z > 2:
                q = QN[i, 1:z - 1, :3]
                q2n.extend((np.sum(q * q, axis=1) / QN[i, 1:z - 1, 3]).tolist())
            ends_q.append(float(np.abs(QN[i, [0, z - 1], :3]).max()))
            rates.extend(tau[i, : z - 1].tolist())
        nh = np.bincount(np.array(Ns), minlength=nk + 1)[: nk + 1]
        q2n = np.array(q2n)
        rates = np.array(rates)
        ens.append({"beta": beta, "nk": nk, "n_chains": n, "seed": seed * n,
                    "z_hist": zh.tolist(), "n_hist": nh.tolist(),
                    "q2_over_n_mean": float(q2n.mean()), "q2_over_n_var": float(q2n.var()),
                    "q2_over_n_count": int(q2n.size), "max_abs_end_q": float(max(ends_q)),
                    "rate_quantiles": {str(q): float(np.quantile(rates, q)) for q in QUANTS},
                    "rate_count": int(rates.size),
                    "sum_n_equals_nk": bool(all(QN[i, : Z[i], 3].sum() == nk for i in range(n)))})
    (HERE / "init_reference.json").write_text(json.dumps({"source": "common/chain.cu:199-283 (compiled, MT19937 seed job_ID*N_cha)", "ensembles": ens}, indent=1))

    # ---- lifetime samplers
    tq = []
    for beta, nk in ((1.0, 25), (1.0, 200), (2.0, 50)):
        for kind in (0, 1):
            n = 200000
            out = np.zeros(n, np.float32)
            R.ref_tau_samples(C.c_float(beta), C.c_float(nk), kind, 12345, n, out.ctypes.data_as(C.c_void_p))
            tq.append({"beta": beta, "nk": nk, "kind": ["f_t", "f_d_t"][kind], "n": n,
                       "tau_quantiles": {str(q): float(np.quantile(out, q)) for q in QUANTS}})
    # ---- GEX tables (separate process per parameter set)
    import subprocess
    exe = HERE.parent.parent / "oracle" / "_ref" / "ref_gex"
    gex = []
    for (a, b, mp, mk, be) in [(1.0, 1.0, 1000.0, 100.0, 1.0), (2.0, 1.0, 1000.0, 100.0, 1.0),
                               (3.0, 2.0, 2000.0, 100.0, 1.0), (1.5, 1.2, 5000.0, 150.0, 2.0)]:
        r = subprocess.run([str(exe), str(a), str(b), str(mp), str(mk), str(be), "100"], capture_output=True,
                           text=True, timeout=600)
        if r.returncode != 0:
            continue
        d = json.loads(r.stdout)
        d.update(a=a, b=b, mp=mp, mk=mk, beta=be)
        gex.append(d)
    (HERE / "gex_reference.json").write_text(json.dumps({"source": "common/gamma.cpp:174-263 (compiled)",
                                                         "rows": gex}))
    (HERE / "tau_reference.json").write_text(json.dumps({"source": "common/pcd_tau.h:67-82 (compiled)", "rows": tq}, indent=1))
    ref_step_fixture()
    print("golden fixtures written to", HERE)


def ref_step_fixture():
    """Reference-kernel trajectories (see the module docstring)."""
    xy = (0.0, 2.0e-3, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0)
    cases = {"eq_nk25_events": dict(nk=25, n=32, seed=11, kappa=(0.0,) * 9, t_end=1000.0, limit=1500),
             "eq_nk25_time": dict(nk=25, n=16, seed=12, kappa=(0.0,) * 9, t_end=120.0, limit=-1),
             "eq_nk200_events": dict(nk=200, n=4, seed=13, kappa=(0.0,) * 9, t_end=1000.0, limit=2000),
             "flow_nk50_events": dict(nk=50, n=16, seed=14, kappa=xy, t_end=1000.0, limit=1000)}
    out = {"cases": np.array(list(cases))}
    for name, c in cases.items():
        flow = any(c["kappa"])
        o = orc.Oracle(nk=c["nk"], n_chains=c["n"], mode=2, seed=c["seed"], kappa=c["kappa"], corr=not flow,
                       sync_dt=1.0, t_end=c["t_end"], corr_p=16, corr_m=2)
        o.init_equilibrium()
        st = o.get_state()
        r = orc.RefStep(o, corr_res=1)
        r.set_chains(st["Z"], st["QN"], st["tau"])
        assert r.run(c["t_end"], c["limit"]) == 0
        b = r.get_state()
        g = {"nk": c["nk"], "n": c["n"], "seed": c["seed"], "kappa": np.array(c["kappa"], np.float32),
             "t_end": c["t_end"], "limit": c["limit"], "Z0": st["Z"], "QN0": st["QN"], "tau0": st["tau"],
             "Z": b["Z"], "QN": b["QN"], "time": b["time"], "events": b["events"]}
        if not flow:
            g["G"] = r.gt()[0]
        for k, v in g.items():
            out[f"{name}/{k}"] = np.asarray(v)
    np.savez_compressed(HERE / "ref_step_reference.npz", **out)


if __name__ == "__main__":
    main()
