"""Headless equivalent of the reference GUI's parameter mapping
(GUI/mainwindow.cpp:556-640, 823-839, GUI/flow.txt): from a probe molecular
weight, a Kuhn-step mass and the model (FSM with its beta, or CFSM) to the
input.dat of a run, and polydisp.dat when a GEX background is given.

- N_K = ceil(M/M_K) (FSM) or the CFSM strand count ceil(M/(0.56 M_K beta)) with
  beta = 1 (mainwindow.cpp:556-562, 583-593);
- equilibrium runs: sync_dt = 1 and t_end = tau_d of the p_cd fit
  (mainwindow.cpp:564-569);
- flow runs: kappa = rate x the flow pattern (flow.txt: shear start-up
  "inception", uniaxial, biaxial, planar extension), t_end = ceil(strain/rate),
  sync_dt = t_end/1000, or 1 below 10 (mainwindow.cpp:570-575, 487-528);
- Wi = rate x tau_d (mainwindow.cpp:823-839).

    python -m gpu_dsm_gb300.setup_run --mw 100 --mk 100 --model CFSM --beta 1 \\
        --flow inception --rate 1e-4 --strain 50 --chains 4096 --dir run1
"""
from __future__ import annotations

import argparse
import math
from pathlib import Path
from typing import Optional, Sequence

FLOW_TYPES = {  # GUI/flow.txt: row-major velocity-gradient transpose per unit rate
    "inception": (0, 1, 0, 0, 0, 0, 0, 0, 0),
    "uniaxial": (-0.5, 0, 0, 0, -0.5, 0, 0, 0, 1),
    "biaxial": (0.5, 0, 0, 0, 0.5, 0, 0, 0, -1),
    "planar": (-1, 0, 0, 0, 0, 0, 0, 0, 1),
}


def tau_d(model: str, n: int, beta: float) -> float:
    """Disentanglement time of the p_cd fit (pcd_tau.h:35-40) as the GUI uses it."""
    if model.upper() == "CFSM":
        return 0.0740131 * n ** 3.18363
    return 0.036 * (beta + 2.0) ** 3.07 * ((n + beta) / (beta + 1.0) - 1.0) ** 3.02


def map_parameters(*, mw_kg_mol: float, mk_g_mol: float, model: str = "CFSM", beta: float = 1.0,
                   n_chains: int = 1000, cd: int = 1, flow: Optional[str] = None, rate: float = 0.0,
                   strain: float = 0.0, gt: bool = True, polydisp: Optional[Sequence[float]] = None) -> dict:
    nk = mw_kg_mol * 1000.0 / mk_g_mol
    if model.upper() == "CFSM":
        n = int(math.ceil(nk / (0.56 * beta)))
        beta_run = 1.0
    elif model.upper() == "FSM":
        n = int(math.ceil(nk))
        beta_run = beta
    else:
        raise ValueError("model must be FSM or CFSM")
    td = tau_d(model, n, beta_run)
    if flow is None:
        kappa = (0.0,) * 9
        sync_dt, t_end = 1.0, td
    else:
        if flow not in FLOW_TYPES or not rate > 0:
            raise ValueError(f"flow must be one of {sorted(FLOW_TYPES)} with rate > 0")
        kappa = tuple(float(v) * rate for v in FLOW_TYPES[flow])
        t_end = float(math.ceil(strain / rate))
        sync_dt = t_end / 1000.0
        if sync_dt < 10:
            sync_dt = 1.0
    return {"beta": beta_run, "nk": n, "n_chains": n_chains, "kappa": kappa, "cd_flag": cd,
            "pd_flag": 1 if polydisp else 0, "eq_type": 1 if (gt and flow is None) else 0,
            "sync_dt": sync_dt, "t_end": t_end, "tau_d": td, "Wi": rate * td if flow else 0.0,
            "polydisp": tuple(polydisp) if polydisp else None}


def write_input(run_dir: Path, p: dict) -> Path:
    """input.dat in the reference's positional format (CLI/input.dat:1-9) and
    polydisp.dat (a b mp Mk) when a GEX background is set."""
    run_dir = Path(run_dir)
    run_dir.mkdir(parents=True, exist_ok=True)
    lines = [f"\t{p['beta']}", f"\t{p['nk']}", f"\t{p['n_chains']}",
             "\t" + "\t".join(f"{k:g}" for k in p["kappa"]), f"\t{p['cd_flag']}", f"\t{p['pd_flag']}",
             f"\t{p['eq_type']}", f"\t{p['sync_dt']:g}", f"\t{p['t_end']:g}"]
    path = run_dir / "input.dat"
    path.write_text("\n".join(lines) + "\n")
    if p.get("polydisp"):
        (run_dir / "polydisp.dat").write_text("".join(f"\t{v:g}\n" for v in p["polydisp"]))
    return path


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--mw", type=float, required=True, help="probe molecular weight (kg/mol)")
    ap.add_argument("--mk", type=float, required=True, help="Kuhn-step molar mass (g/mol)")
    ap.add_argument("--model", default="CFSM", choices=["CFSM", "FSM"])
    ap.add_argument("--beta", type=float, default=1.0, help="FSM entanglement activity")
    ap.add_argument("--chains", type=int, default=1000)
    ap.add_argument("--no-cd", action="store_true")
    ap.add_argument("--flow", choices=sorted(FLOW_TYPES))
    ap.add_argument("--rate", type=float, default=0.0, help="deformation rate (1/tau_K)")
    ap.add_argument("--strain", type=float, default=0.0)
    ap.add_argument("--polydisp", type=float, nargs=4, metavar=("A", "B", "MP", "MK"))
    ap.add_argument("--dir", default=".")
    a = ap.parse_args(argv)
    p = map_parameters(mw_kg_mol=a.mw, mk_g_mol=a.mk, model=a.model, beta=a.beta, n_chains=a.chains,
                       cd=0 if a.no_cd else 1, flow=a.flow, rate=a.rate, strain=a.strain, polydisp=a.polydisp)
    path = write_input(Path(a.dir), p)
    print(f"{path}: N_K={p['nk']} beta={p['beta']} t_end={p['t_end']:g} sync_dt={p['sync_dt']:g} "
          f"tau_d={p['tau_d']:.4g}" + (f" Wi={p['Wi']:.4g}" if a.flow else ""))
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
