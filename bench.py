#!/usr/bin/env python3
"""Benchmark: kMC events/s of the N_K=200 monodisperse melt on one GB300.

Workload (the headline configuration): 65536 chains, N_K=200 Kuhn steps,
beta=1, constraint dynamics on, equilibrium initial state, multi-tau G(t)
correlator (p=64, m=8, levels for t_end=1e7 tau_K, sample every 1 tau_K) on
the three shear stresses.  A "step" advances the whole ensemble by a window
of --window tau_K (default 500) in steady state; inputs are already resident in
HBM.  The ensemble state (~260 MB conformations + ~590 MB correlator) exceeds
the 129 MB L2, so no explicit L2 flush is needed between steps.

Also reported:
  e2e           same metric through the C ABI with the conformations uploaded
                from pinned host memory and read back every step (plus G(t))
  roofline      SM-issue bound of the step kernel: lane-ops per event
                L_eq(Z) = 2(Z-1) + 152 against 152 SMs x 128 lanes x f_max
  cpu_baseline  the oracle (CPU restatement of the reference path) on the
                host cores, bounded sample of the same workload
  gt_err_vs_fp64  the CPU leg also checks the GPU's results against the FP64
                transcription of the reference path (oracle mode 1) on the same
                chains and random streams: G(t) of 512 chains of the headline
                ensemble, sigma_xy of shear samples, G(t) of served requests
  --impl reference  times that CPU restatement as the reference arm
  --gpus N      without a torchrun environment, starts N ranks itself
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "kMC events/s on 1 GB300 (N_K=200); serve p50/p99 vs plain at G(t) err<=1%"
UNIT = "events/s"
NK, BETA = 200, 1.0
N_CHAINS = 65536
T_END_RUN, SAMPLE_DT, CORR_P, CORR_M = 1.0e7, 1.0, 64, 8


def config(window: float, n_gpus: int) -> dict:
    return {"workload": f"equilibrium monodisperse melt: {N_CHAINS} chains x N_K={NK}, beta={BETA}, CD on, "
                        f"G(t) multi-tau p={CORR_P} m={CORR_M} over xy/yz/xz (levels for t_end=1e7, dt=1)",
            "n_chains_per_gpu": N_CHAINS, "nk": NK, "beta": BETA, "window_tau_per_step": window,
            "l2": "inputs larger than L2 (state ~0.85 GB per GPU); no flush",
            "parallelism": f"chains sharded over {n_gpus} GPU(s), G(t) sums all-reduced at output"}


# ---------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int = 0):
        self.device = device
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except FileNotFoundError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------- CPU legs
def cpu_sample(target_s: float, threads: int = 0, n: int = 256):
    """Time the oracle (FP32 mirror, OpenMP over chains) on a bounded sample of the
    workload: n chains of N_K=200 from the equilibrium state, advanced by a window
    sized to ~target_s of CPU time after a short calibration."""
    from oracle import oracle as orc

    orc.build()
    o = orc.Oracle(nk=NK, n_chains=n, seed=1, corr=True, sync_dt=SAMPLE_DT, t_end=T_END_RUN, corr_p=CORR_P,
                   corr_m=CORR_M, threads=threads)
    o.init_equilibrium()
    t0 = time.perf_counter()
    ev = o.run(2.0)
    dt = time.perf_counter() - t0
    rate = ev / max(dt, 1e-6)
    window = max(2.0, min(2000.0, target_s * rate / (n * 42.6)))
    t0 = time.perf_counter()
    ev = o.run(2.0 + window)
    dt = time.perf_counter() - t0
    return {"value": ev / dt, "unit": UNIT, "cores": o.threads, "kind": "port",
            "sample": f"{n} chains x {window:.0f} tau_K of the N_K=200 workload (oracle FP32 mirror, "
                      f"{ev} events in {dt:.1f} s)"}, o


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    # whole run ~90 s of CPU time: a short calibration, then K+W steps of ~equal size
    per_step = max(2.0, 80.0 / max(1, args.steps + args.warmup))
    base, o = cpu_sample(3.0)
    n = o.n
    t_cur = 2.0 + float(base["sample"].split(" x ")[1].split(" ")[0])
    rates = []
    window = max(1.0, per_step * base["value"] / (n * 42.6))
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        ev = o.run(t_cur + window)
        dt = time.perf_counter() - t0
        t_cur += window
        if i >= args.warmup:
            rates.append((ev, dt))
    ev = sum(e for e, _ in rates)
    dt = sum(d for _, d in rates)
    v = ev / dt
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * dt / max(1, args.steps), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic equilibrium melt",
            "config": config(window, args.gpus), "impl": "reference",
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": o.threads, "kind": "port",
                             "sample": f"{n} chains x {window:.0f} tau_K per step of the N_K=200 workload "
                                       f"(oracle, the reference's chain-step logic restated in C++/OpenMP; the "
                                       f"reference GPU code does not compile with CUDA 13)"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


# ---------------------------------------------------------------- GPU leg
def measured_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        return json.loads(p.read_text())
    return {}


def profile_traffic() -> dict:
    p = ROOT / "profiles" / "step_kernel_traffic.json"
    return json.loads(p.read_text()) if p.exists() else {}


def fp64_accuracy(args, device: int, shear: dict | None, serve: dict | None) -> dict:
    """Part of the CPU leg: the FP64 transcription (oracle mode 1) on chains the
    GPU also runs, with the same random streams (Philox keyed by chain and
    event), compared with the GPU's results against the FP64 estimate's own
    chain-to-chain error (oracle.gt_error_vs_fp64):
      headline  G(t) of chains 30000-30511 of the headline ensemble over 500 tau_K;
      shear     sigma_xy of 256 chains at Wi 0.1, 1, 10 and 100 (N_K=100) at
                five outputs, deviation in units of sigma; with the FP64
                sigma_xy at the last output and its standard error, for 256
                chains and scaled to the 32768 chains per Wi of the timed leg;
      serve     G(t) of the two cheapest G(t) requests of the served stream,
                re-run on the CPU with the request's parameters."""
    import gpu_dsm_gb300 as dsm
    from oracle import oracle as orc

    out = {}
    kw = dict(nk=NK, n_chains=512, beta=BETA, sync_dt=SAMPLE_DT, t_end=T_END_RUN, corr_p=CORR_P, corr_m=CORR_M,
              seed=1, chain_offset=30000)
    g = dsm.Ensemble(eq_type=1, device=device, **kw)
    f = orc.Oracle(corr=True, mode=1, **kw)
    g.init_equilibrium()
    f.init_equilibrium()
    g.advance(500.0)
    f.run(500.0)
    out["headline"] = {**orc.gt_error_vs_fp64(g.gt_raw()[0], f),
                       "sample": "chains 30000-30511 of the headline ensemble, 500 tau_K, G(t) sums"}
    g.close()
    if shear is not None and "failed" not in shear:
        tau_d = dsm.pcd(1.0, 100)["tau_d"]
        rows = []
        for wi in (0.1, 1.0, 10.0, 100.0):
            kap = (0.0, wi / tau_d, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0)
            skw = dict(nk=100, n_chains=256, kappa=kap, seed=4, stream=3)
            ge = dsm.Ensemble(sync_dt=100.0, t_end=5.0e5, device=device, **skw)
            fe = orc.Oracle(mode=1, **skw)
            ge.init_equilibrium()
            fe.init_equilibrium()
            worst = 0.0
            for w in range(1, 6):
                ge.advance(100.0 * w)
                fe.run(100.0 * w)
                sg = ge.stress()[0][3]
                sf = fe.stress()[0][3]
                st = fe.get_state()
                q = st["QN"].astype(np.float64)
                idx = np.arange(q.shape[1])[None, :] < st["Z"][:, None]
                per = -3.0 * np.where(idx, q[:, :, 0] * q[:, :, 1] / np.where(idx, q[:, :, 3], 1.0), 0.0).sum(axis=1)
                worst = max(worst, abs(sg - sf) / (per.std(ddof=1) / math.sqrt(len(per))))
            ge.close()
            sd = float(per.std(ddof=1))
            rows.append({"wi": wi, "dev_sigma": worst, "sigma_xy_fp64_at_500": float(sf),
                         "se_256_chains": sd / math.sqrt(len(per)),
                         "se_at_timed_leg_chains": sd / math.sqrt(args.shear_chains)})
        shear["stress_err_vs_fp64"] = {"rows": rows, "sample": "256 chains, N_K=100, outputs every 100 tau_K "
                                       "to 500 tau_K; |sigma_xy(GPU) - sigma_xy(FP64)| / sigma of the FP64 "
                                       "estimate; consistent when below 3 sqrt(2). se_at_timed_leg_chains: "
                                       "the chain-to-chain error of sigma_xy_per_window in the timed leg"}
        out["shear"] = shear["stress_err_vs_fp64"]
    if serve is not None and serve.get("_samples"):
        rows = []
        for r, gp in serve.pop("_samples"):
            fo = orc.Oracle(nk=r["nk"], n_chains=r["n_chains"], beta=r["beta"], seed=r["seed"], stream=r["stream"],
                            corr=True, sync_dt=r["sync_dt"], t_end=r["t_end"], corr_p=r["corr_p"],
                            corr_m=r["corr_m"], mode=1)
            fo.init_equilibrium()
            fo.run(r["t_end"])
            rows.append({**orc.gt_points_error_vs_fp64(gp, fo),
                         "request": {k: r[k] for k in ("nk", "beta", "n_chains", "t_end")}})
        serve["gt_err_vs_fp64"] = rows
        out["serve"] = rows
    return out


def latency_probe(args, device: int, f_hz: float, tiles_per_sm: int, value: float) -> dict:
    """Latency model of the step kernel: 304 chains of the headline workload
    run as one warp (two 16-lane chain tiles) per block, so that each SM holds
    a single warp; their events per second give the critical-path cycles per
    event of a chain that waits for nothing but its own dependencies.  The
    bound is every resident chain tile of the headline schedule running at that
    speed; frac = achieved / bound."""
    import gpu_dsm_gb300 as dsm

    n = 2 * 152
    e = dsm.Ensemble(beta=BETA, nk=NK, n_chains=n, eq_type=1, sync_dt=SAMPLE_DT, t_end=T_END_RUN, seed=9,
                     device=device, corr_p=CORR_P, corr_m=CORR_M, lanes_per_chain=16, warps_per_block=1)
    e.init_equilibrium()
    e.advance(50.0)
    ev = e.advance(2050.0)
    lw = e.last_window()
    e.close()
    rate = ev / (lw["kernel_ms"] / 1e3)
    cyc = f_hz * n / rate
    bound = 152 * tiles_per_sm * f_hz / cyc
    return {"critical_path_cycles_per_event": cyc, "probe": f"{n} chains, 1 warp (2 chain tiles) per SM, "
            f"{ev} events, {lw['grid']} blocks", "resident_chain_tiles_per_sm": tiles_per_sm,
            "achieved": value / 1e9, "peak": bound / 1e9, "unit": "Gevents/s", "frac": value / bound,
            "cycles_per_event_at_load": 152 * tiles_per_sm * f_hz / value,
            "note": "peak = 152 SMs x resident chain tiles x clock / critical-path cycles per event"}


def spawn_ranks(args) -> int:
    """--gpus N outside torchrun: start N ranks with torch.distributed.run on
    127.0.0.1 (one process per GPU) and pass rank 0's JSON line through."""
    import socket

    with socket.socket() as so:
        so.bind(("127.0.0.1", 0))
        port = so.getsockname()[1]
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={args.gpus}",
           "--master-addr", "127.0.0.1", "--master-port", str(port), str(ROOT / "bench.py"), *sys.argv[1:]]
    return subprocess.run(cmd).returncode


def run_gpu(args):
    import torch
    import gpu_dsm_gb300 as dsm
    from gpu_dsm_gb300 import build as native

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world != args.gpus:
        raise SystemExit(f"bench: --gpus {args.gpus} but WORLD_SIZE={world}")
    comm = {"backend": None, "world_size": 1}
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
        comm = {"backend": dist.get_backend(), "world_size": dist.get_world_size()}
        if comm["world_size"] != args.gpus:
            raise SystemExit(f"bench: NCCL communicator of {comm['world_size']} ranks, --gpus {args.gpus}")
    if rank == 0:
        native.build()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.set_device(local)

    # one ensemble of world x N_CHAINS chains sharded over the ranks (weak
    # scaling): rank r holds chains [r*N_CHAINS, (r+1)*N_CHAINS), random streams
    # keyed by global chain id
    ens = dsm.Ensemble(beta=BETA, nk=NK, n_chains=N_CHAINS, eq_type=1, sync_dt=SAMPLE_DT, t_end=T_END_RUN,
                       seed=1, device=local, corr_p=CORR_P, corr_m=CORR_M, lanes_per_chain=args.lanes,
                       chain_offset=rank * N_CHAINS)
    ens.init_equilibrium()
    t = 0.0
    for _ in range(args.warmup):
        t += args.window
        ens.advance(t)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clk = ClockSampler(local)
    clk.start()
    events, kms = 0, 0.0
    t0 = time.perf_counter()
    for _ in range(args.steps):
        t += args.window
        events += ens.advance(t)
        kms += ens.last_window()["kernel_ms"]
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    wall = time.perf_counter() - t0
    clocks = clk.stop()
    lw = ens.last_window()
    sched = ens.schedule()
    launches_per_step = max(1, len(sched))  # size classes + overflow launch, or one launch
    heads, qn, tau = ens.get_chains()
    zmean = float(heads["Z"].mean())
    gt_points = None
    if world > 1:
        import torch.distributed as dist
        from gpu_dsm_gb300 import sharded
        # the exchange step: global G(t) from the per-rank correlator sums
        _, g_all = sharded.sharded_gt(ens, n_total=world * N_CHAINS, p=CORR_P, m=CORR_M, sync_dt=SAMPLE_DT,
                                      t_end=T_END_RUN)
        gt_points = int(len(g_all))
        tt = torch.tensor([kms, float(events)], dtype=torch.float64, device="cuda")
        mx = tt.clone()
        dist.all_reduce(mx, op=dist.ReduceOp.MAX)
        dist.all_reduce(tt, op=dist.ReduceOp.SUM)
        kms_max, events_all = float(mx[0]), int(tt[1])
    else:
        kms_max, events_all = kms, events
    value = events_all / (kms_max / 1e3)

    # ---- e2e through the C ABI with host buffers (pinned), every step, on
    # every rank (each its own shard); whole-job events over the slowest rank
    e2e = None
    if args.e2e_steps > 0:
        cap = ens.z_max
        h_heads = torch.empty(N_CHAINS * 16, dtype=torch.uint8, pin_memory=True)
        h_qn = torch.empty(N_CHAINS * cap * 4, dtype=torch.float32, pin_memory=True)
        h_tau = torch.empty(N_CHAINS * cap, dtype=torch.float32, pin_memory=True)
        hv = h_heads.numpy().view(dsm.api.HEAD_DTYPE)
        qv = h_qn.numpy().reshape(N_CHAINS, cap, 4)
        tv = h_tau.numpy().reshape(N_CHAINS, cap)
        hv[:] = heads
        hv["time"] = 0.0
        qv[:] = qn
        tv[:] = tau
        ens2 = dsm.Ensemble(beta=BETA, nk=NK, n_chains=N_CHAINS, eq_type=1, sync_dt=SAMPLE_DT,
                            t_end=T_END_RUN, seed=2, device=local, corr_p=CORR_P, corr_m=CORR_M,
                            chain_offset=rank * N_CHAINS)
        # results come back into pinned buffers of their own
        o_heads = torch.empty(N_CHAINS * 16, dtype=torch.uint8, pin_memory=True)
        o_qn = torch.empty(N_CHAINS * cap * 4, dtype=torch.float32, pin_memory=True)
        o_tau = torch.empty(N_CHAINS * cap, dtype=torch.float32, pin_memory=True)
        outs = (o_heads.numpy().view(dsm.api.HEAD_DTYPE), o_qn.numpy().reshape(N_CHAINS, cap, 4),
                o_tau.numpy().reshape(N_CHAINS, cap))
        ev_e, t_e = 0, 0.0
        npts = 0
        for i in range(args.e2e_steps + 1):
            torch.cuda.synchronize()
            if world > 1:
                torch.distributed.barrier()
            s0 = time.perf_counter()
            ens2.set_chains(hv, qv, tv)
            ev = ens2.advance(args.window)
            ens2.get_chains(out=outs)
            tg, g = ens2.gt()
            torch.cuda.synchronize()
            s1 = time.perf_counter()
            npts = len(g)
            if i > 0:  # first e2e step is a warm-up
                ev_e += ev
                t_e += s1 - s0
        h2d = (N_CHAINS * 16 + N_CHAINS * cap * 20) * world
        d2h = (N_CHAINS * 16 + N_CHAINS * cap * 20 + npts * 8) * world
        if world > 1:
            import torch.distributed as dist
            et = torch.tensor([float(ev_e)], dtype=torch.float64, device="cuda")
            tt_e = torch.tensor([t_e], dtype=torch.float64, device="cuda")
            dist.all_reduce(et, op=dist.ReduceOp.SUM)
            dist.all_reduce(tt_e, op=dist.ReduceOp.MAX)
            ev_e, t_e = int(et.item()), float(tt_e.item())
        e2e = {"value": ev_e / t_e, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
               "steps": args.e2e_steps, "host_buffers": "pinned (torch pin_memory)",
               "calls": "dsm_set_chains + dsm_advance + dsm_get_chains + dsm_gt"}
        ens2.close()

    # ---- roofline: SM-issue bound (lane-ops per event) + HBM secondary
    peaks = measured_peaks()
    f_max = float(peaks.get("sm_max_mhz", 2070.0)) * 1e6
    n_sm = 152
    l_eq = 2.0 * (zmean - 1.0) + 152.0
    peak_lane = n_sm * 128 * f_max
    achieved_lane = value / world * l_eq
    per_launch_events = events / max(1, args.steps)
    tr = profile_traffic()
    traffic = None
    if tr.get("bytes_per_event"):
        traffic = float(tr["bytes_per_event"]) * per_launch_events
    roof = {"bound": "sm_issue", "achieved": achieved_lane / 1e9, "peak": peak_lane / 1e9, "unit": "Glane-op/s",
            "frac": achieved_lane / peak_lane, "traffic": traffic,
            "per_unit": f"L_eq(Z)=2(Z-1)+152 lane-ops per kMC event at <Z>={zmean:.1f}",
            "peak_source": "152 SMs x 128 lanes x sm_max_mhz of MEASURED_PEAKS.json (of measured clock)"}
    if peaks.get("hbm_gbs"):
        # algorithmic HBM bytes per step: chain state in + out once per window, correlator levels
        bytes_chain = N_CHAINS * (2 * (zmean * 20 + 64) + 2 * (CORR_P * 12 + 44) + CORR_P * 16)
        samples = N_CHAINS * args.window / SAMPLE_DT
        lvl_bytes = samples * sum((1.0 / CORR_M ** k) * (CORR_P * 12 + 12 + (CORR_P - CORR_P // CORR_M) * 16 + 44)
                                  for k in range(1, 7))
        gbs = (bytes_chain + lvl_bytes) / (kms / args.steps / 1e3) / 1e9
        roof["hbm_secondary"] = {"achieved": gbs, "peak": float(peaks["hbm_gbs"]), "unit": "GB/s",
                                 "frac": gbs / float(peaks["hbm_gbs"]), "note": "of measured"}
    if tr.get("warp_instructions_per_event"):
        # issue slots: the kernel is latency-bound, so the share of warp-scheduler
        # issue slots it fills (events/s x warp-instructions per event from the
        # ncu capture, against 4 schedulers x 152 SMs x clock) says how busy the SMs are
        ipe = float(tr["warp_instructions_per_event"])
        peak_issue = n_sm * 4 * f_max
        roof["issue_secondary"] = {"achieved": value / world * ipe / 1e9, "peak": peak_issue / 1e9,
                                   "unit": "Gwarp-inst/s", "frac": value / world * ipe / peak_issue,
                                   "per_unit": f"{ipe:g} warp-instructions per kMC event (ncu)",
                                   "note": "of measured clock"}

    if rank == 0 and not args.no_latency:
        try:
            tiles = int(lw["blocks_per_sm"]) * (128 // max(16, int(sched[0]["lanes"]) if sched else 16))
            roof["latency_secondary"] = latency_probe(args, local, float(clocks.get("sm_mhz") or 2070.0) * 1e6,
                                                      tiles, value / world)
        except Exception as e:  # reported, never silently replaced
            roof["latency_secondary"] = {"failed": repr(e)}

    if rank != 0:
        ens.close()
        torch.distributed.destroy_process_group()
        return 0
    serve = shear = poly = None
    if world == 1:
        ens.close()
    if not args.no_poly and world == 1:
        try:
            poly = run_poly(args, local)
        except Exception as e:  # reported, never silently replaced
            poly = {"failed": repr(e)}
    if not args.no_shear and world == 1:
        try:
            shear = run_shear(args, local)
        except Exception as e:  # reported, never silently replaced
            shear = {"failed": repr(e)}
    if not args.no_serve and world == 1:
        try:
            serve = run_serve(args, local)
        except Exception as e:  # reported, never silently replaced
            serve = {"failed": repr(e)}
    cpu = None
    acc = None
    if not args.no_cpu:
        try:
            cpu, _ = cpu_sample(args.cpu_seconds)
        except Exception as e:  # the baseline is reported, never a fallback
            cpu = {"value": None, "unit": UNIT, "cores": 0, "kind": "port", "sample": f"failed: {e}"}
        if world == 1:
            try:
                acc = fp64_accuracy(args, local, shear, serve)
            except Exception as e:  # reported, never silently replaced
                acc = {"failed": repr(e)}
    if isinstance(serve, dict):
        serve.pop("_samples", None)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": kms_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+i64", "data": "synthetic equilibrium melt",
            "config": config(args.window, world), "roofline": roof, "cpu_baseline": cpu, "e2e": e2e,
            "clocks": clocks, "gpu_launches": args.steps * launches_per_step, "shear": shear, "poly": poly,
            "serve": serve, "gt_err_vs_fp64": (acc or {}).get("headline", acc),
            "comm": comm,
            "detail": {"events": events_all, "wall_s": wall, "kernel_ms_total": kms, "mean_Z": zmean,
                       "sharded_gt_points": gt_points,
                       "grid": lw["grid"], "blocks_per_sm": lw["blocks_per_sm"], "schedule": sched}}
    print(json.dumps(line))
    ens.close()
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


# ---------------------------------------------------------------- shear start-up
def run_shear(args, device: int = 0) -> dict:
    """Steady shear start-up: four ensembles of 32768 chains, N_K=100, beta=1,
    kappa_xy = Wi / tau_d for Wi in {0.1, 1, 10, 100}, advanced together by
    dsm_advance_batch (one persistent launch) with a stress output per window
    of t_end/1000 = 500 tau_K (t_end = 5e5).  A bounded sample: the first
    --shear-windows output windows after equilibrium start."""
    import gpu_dsm_gb300 as dsm

    nk, n, t_end = 100, args.shear_chains, 5.0e5
    dt_out = args.shear_window if args.shear_window > 0 else t_end / 1000.0
    tau_d = dsm.pcd(1.0, nk)["tau_d"]
    ens = [dsm.Ensemble(nk=nk, n_chains=n, beta=1.0, kappa=(0.0, wi / tau_d, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0),
                        sync_dt=dt_out, t_end=t_end, seed=4, stream=k, device=device)
           for k, wi in enumerate((0.1, 1.0, 10.0, 100.0))]
    for e in ens:
        e.init_equilibrium()
    ev_tot, secs, series, zs = 0, 0.0, [], []
    t = 0.0
    for w in range(args.shear_windows):
        t += dt_out
        t0 = time.perf_counter()
        ev = dsm.advance_batch(ens, t)
        secs += time.perf_counter() - t0
        ev_tot += int(np.sum(ev))
        st = [e.stress()[0] for e in ens]
        series.append([float(x[3]) for x in st])
        zs.append(float(np.mean([x[7] for x in st])))
    for e in ens:
        e.close()
    rate = ev_tot / secs
    # flow roofline: every pair rate is recomputed after the deformation, so
    # L_flow(Z) = L_eq(Z) + 9 Z (deformation) + 40 (Z - 1) (pair rates)
    zmean = float(np.mean(zs))
    l_flow = 2.0 * (zmean - 1.0) + 152.0 + 9.0 * zmean + 40.0 * (zmean - 1.0)
    f_max = float(measured_peaks().get("sm_max_mhz", 2070.0)) * 1e6
    peak_lane = 152 * 128 * f_max
    roof = {"bound": "sm_issue", "achieved": rate * l_flow / 1e9, "peak": peak_lane / 1e9, "unit": "Glane-op/s",
            "frac": rate * l_flow / peak_lane,
            "per_unit": f"L_flow(Z)=2(Z-1)+152+9Z+40(Z-1) lane-ops per kMC event at <Z>={zmean:.1f}",
            "peak_source": "152 SMs x 128 lanes x sm_max_mhz of MEASURED_PEAKS.json (of measured clock)"}
    return {"workload": f"4 x {n} chains, N_K=100, beta=1, shear Wi {{0.1,1,10,100}}, kappa_xy=Wi/tau_d, "
                        f"tau_d={tau_d:.4g}, output every {dt_out:g} tau_K",
            "windows": args.shear_windows, "events": ev_tot, "events_per_s": rate, "wall_s": secs,
            "sigma_xy_per_window": series, "roofline": roof,
            "timing": "host wall clock around dsm_advance_batch (launch + window + stress readback)"}


# ---------------------------------------------------------------- polydisperse melt
def run_poly(args, device: int = 0) -> dict:
    """Batched polydisperse melt: 262144 chains, N_K log-normal (mean 150,
    PDI 1.5 = exp(sigma^2), clipped to [10, 2000], seed 7), beta=1, G(t)
    p=64 m=8 (levels for t_end=1e6).  Size classes as concurrent persistent
    launches or as one carved launch, the schedule and form chosen by the online
    autotuner on --poly-tune-window windows,
    then --poly-windows timed windows of --poly-window tau_K (default 4 x 250,
    1e3 tau_K as for the monodisperse workload) in one dsm_advance_series call."""
    import gpu_dsm_gb300 as dsm

    n = args.poly_chains
    rng = np.random.default_rng(7)
    s2 = math.log(1.5)
    nkc = np.clip(np.round(np.exp(rng.normal(math.log(150.0) - s2 / 2, math.sqrt(s2), size=n))), 10, 2000)
    nkc = nkc.astype(np.int32)
    e = dsm.Ensemble(nk=int(nkc.max()), n_chains=n, nk_chain=nkc, eq_type=1, sync_dt=1.0, t_end=1.0e6, corr_p=64,
                     corr_m=8, seed=7, device=device)
    e.init_equilibrium()
    e.advance(args.poly_tune_window)
    best = e.autotune(args.poly_tune_window)
    if args.poly_form >= 0:  # force the class form after tuning (0 concurrent launches, 1 carved launch)
        e.set_class_form(args.poly_form)
    form = e.class_form()
    ev, _ = e.advance_series(args.poly_window, args.poly_windows)
    ms = e.last_window()["kernel_ms"]
    sched = e.schedule()
    e.close()
    return {"workload": f"{n} chains, N_K log-normal mean 150 PDI 1.5 in [10, 2000] (mean {nkc.mean():.1f}, "
                        f"max {int(nkc.max())}), beta=1, G(t) p=64 m=8",
            "events_per_s": ev / (ms / 1e3), "events": int(ev), "kernel_ms": ms,
            "windows": args.poly_windows, "window_tau": args.poly_window, "autotune": best, "schedule": sched,
            "class_form": "one carved launch (large, middle, small) + huge class beside it" if form == 1
                          else "concurrent launches, one per class",
            "timing": "CUDA events around the windows of one dsm_advance_series call (size-class launches + "
                      "overflow launch per window, issued without host synchronisation)"}


# ---------------------------------------------------------------- serving
def serve_stream(n: int, seed: int, t_scale: float):
    """Rheology request stream: N_K log-uniform [20, 500], beta in {0.5, 1, 2},
    1024-65536 chains log-uniform, half equilibrium G(t) (sample every tau_K,
    p=16, m=2), half steady shear at Wi log-uniform [0.1, 100]
    (kappa_xy = Wi / tau_d(beta, N_K)) with 100 stress outputs; t_end
    log-uniform [1e4, 1e6] tau_K times t_scale."""
    import gpu_dsm_gb300 as dsm

    rng = np.random.default_rng(seed)
    lu = lambda a, b: float(np.exp(rng.uniform(math.log(a), math.log(b))))
    reqs = []
    for i in range(n):
        nk = int(round(lu(20, 500)))
        beta = float(rng.choice([0.5, 1.0, 2.0]))
        n_cha = int(round(lu(1024, 65536)))
        shear = bool(rng.integers(0, 2))
        wi = lu(0.1, 100.0)
        t_end = lu(1.0e4, 1.0e6) * t_scale
        r = dict(nk=nk, beta=beta, n_chains=n_cha, t_end=t_end, seed=seed * 1000 + i, stream=i)
        if shear:
            kxy = wi / dsm.pcd(beta, nk)["tau_d"]
            r.update(kappa=(0.0, kxy, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0), sync_dt=t_end / 100.0)
        else:
            r.update(eq_type=1, sync_dt=1.0, corr_p=16, corr_m=2)
        reqs.append(r)
    return reqs


def prior_events(r) -> float:
    return (0.2 * r["nk"] + 2.0) * r["n_chains"] * r["t_end"]


def serve_once(reqs, arrivals, *, max_active, chunk_s, device, policy="fcfs", overlap=1.0, bypass=0.2):
    import gpu_dsm_gb300 as dsm

    srv = dsm.Server(device=device, max_active=max_active, chunk_s=chunk_s, policy=policy, overlap=overlap,
                     bypass=bypass)
    ids = []
    t0 = time.perf_counter()
    for r, a in zip(reqs, arrivals):
        d = t0 + a - time.perf_counter()
        if d > 0:
            time.sleep(d)
        ids.append(srv.submit(**r))
    srv.wait_all(3600.0)
    wall = time.perf_counter() - t0
    st = [srv.status(i) for i in ids]
    out = []
    for r, i, x in zip(reqs, ids, st):
        if x["state"] != dsm.api.REQ_DONE:
            out.append(np.zeros(0, np.float32))
            continue
        out.append(srv.result_gt(i)[1] if r.get("eq_type") == 1 else srv.result_stress(i)[1])
    errors = sorted({x.get("error", "") for x in st if x["state"] != dsm.api.REQ_DONE})
    tot = srv.stats()
    srv.close()
    lat = np.array([x["latency_s"] for x in st])
    failed = sum(1 for x in st if x["state"] != dsm.api.REQ_DONE)
    ev = sum(x["events"] for x in st)
    return {"p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
            "mean_s": float(lat.mean()), "events_per_s": ev / wall, "makespan_s": wall, "events": int(ev),
            "failed": failed, "errors": errors[:5], "chunks": tot["chunks"], "peak_active": tot["peak_active"],
            "peak_bytes": tot["peak_bytes"], "busy_s": tot["busy_s"], "setup_s": tot["setup_s"],
            "finish_s": tot["finish_s"]}, out


def run_serve(args, device: int = 0) -> dict:
    """Served (continuous batching) against plain (one request at a time, one
    launch per request or output interval) on the same Poisson arrivals.
    Offered load = 1.2 x the plain form's throughput, measured first on a
    calibration stream (seed 12) submitted at once."""
    cal = serve_stream(args.serve_cal, 12, args.serve_scale)
    c, _ = serve_once(cal, [0.0] * len(cal), max_active=1, chunk_s=-1.0, device=device)
    reqs = serve_stream(args.serve_requests, 11, args.serve_scale)
    est = np.array([prior_events(r) for r in reqs])
    cal_prior = sum(prior_events(r) for r in cal)
    # plain throughput in prior-estimated events per second of wall time
    plain_rate = cal_prior / c["makespan_s"]
    lam = 1.2 * plain_rate / est.mean()
    rng = np.random.default_rng(11)
    arrivals = np.cumsum(rng.exponential(1.0 / lam, size=len(reqs)))
    arrivals -= arrivals[0]
    served, out_s = serve_once(reqs, arrivals, max_active=0, chunk_s=args.serve_chunk, device=device, policy="fcfs")
    plain, out_p = serve_once(reqs, arrivals, max_active=1, chunk_s=-1.0, device=device)
    others = {}
    for spec in args.serve_policies.split(","):
        # policy[:overlap[:bypass]]
        if not spec:
            continue
        f = spec.split(":")
        pol = f[0]
        ov = float(f[1]) if len(f) > 1 else 1.0
        bp = float(f[2]) if len(f) > 2 else 0.2
        others[spec], _ = serve_once(reqs, arrivals, max_active=0, chunk_s=args.serve_chunk, device=device,
                                     policy=pol, overlap=ov, bypass=bp)
    err = 0.0
    for r, a, b in zip(reqs, out_s, out_p):
        if r.get("eq_type") == 1 and len(a) and len(b):
            err = max(err, float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-30)))
    # the two cheapest G(t) requests, for the CPU leg's check against the FP64 oracle
    cheap = sorted((prior_events(r) * r["nk"], i) for i, r in enumerate(reqs)
                   if r.get("eq_type") == 1 and len(out_s[i]))[:2]
    return {"requests": len(reqs), "t_end_scale": args.serve_scale, "arrival_rate_per_s": lam,
            "offered_load_vs_plain": 1.2, "chunk_s": args.serve_chunk, "served": served, "plain": plain,
            "other_policies": others,
            "policies": "served: first come first served with backfill (stream priority by age, running "
                        "requests up to 1 GPU of chain slots, requests under 0.2 chunk of the GPU start at "
                        "once); plain: one request at a time, one launch per request / flow output",
            "p99_speedup": plain["p99_s"] / served["p99_s"], "p50_speedup": plain["p50_s"] / served["p50_s"],
            "throughput_ratio": served["events_per_s"] / plain["events_per_s"],
            "gt_max_rel_diff_served_vs_plain": err,
            "_samples": [(reqs[i], out_s[i]) for _, i in cheap],
            "stream": "Poisson arrivals (seed 11); N_K log-uniform [20,500], beta {0.5,1,2}, 1024-65536 chains, "
                      "50% G(t) / 50% shear Wi log-uniform [0.1,100], t_end log-uniform [1e4,1e6] x t_end_scale"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--window", type=float, default=500.0, help="tau_K advanced per step")
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--e2e-steps", type=int, default=6)
    ap.add_argument("--no-latency", action="store_true", help="skip the latency-model probe")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--chains", type=int, default=65536, help="chains per GPU (65536 = headline workload)")
    ap.add_argument("--lanes", type=int, default=0, help="lanes per chain (16 or 32; 0 = library default)")
    ap.add_argument("--no-serve", action="store_true", help="skip the serving-stream leg")
    ap.add_argument("--no-shear", action="store_true", help="skip the shear start-up leg")
    ap.add_argument("--shear-only", action="store_true", help="run only the shear start-up leg")
    ap.add_argument("--shear-windows", type=int, default=6)
    ap.add_argument("--no-poly", action="store_true", help="skip the polydisperse leg")
    ap.add_argument("--poly-only", action="store_true", help="run only the polydisperse leg")
    ap.add_argument("--poly-chains", type=int, default=262144)
    ap.add_argument("--poly-window", type=float, default=250.0, help="tau_K per timed polydisperse window")
    ap.add_argument("--poly-windows", type=int, default=4)
    ap.add_argument("--poly-tune-window", type=float, default=5.0, help="tau_K per autotuner candidate window")
    ap.add_argument("--poly-form", type=int, default=-1,
                    help="size-class form after autotuning: -1 the autotuner's, 0 concurrent launches, 1 carved launch")
    ap.add_argument("--shear-chains", type=int, default=32768, help="chains per shear ensemble")
    ap.add_argument("--shear-window", type=float, default=0.0, help="tau_K per output window (0: t_end/1000)")
    ap.add_argument("--serve-only", action="store_true", help="run only the serving-stream leg")
    ap.add_argument("--serve-requests", type=int, default=200)
    ap.add_argument("--serve-cal", type=int, default=16)
    ap.add_argument("--serve-scale", type=float, default=1.0e-3, help="t_end multiplier of the request stream")
    ap.add_argument("--serve-chunk", type=float, default=0.05, help="target chunk duration of the served form (s)")
    ap.add_argument("--serve-policies", default="", help="other serving policies to run too (equal_pace,fcfs_strict)")
    args = ap.parse_args()
    global N_CHAINS
    N_CHAINS = args.chains
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        return spawn_ranks(args)
    if args.poly_only:
        from gpu_dsm_gb300 import build as native
        native.build()
        print(json.dumps({"poly": run_poly(args)}))
        return 0
    if args.shear_only:
        from gpu_dsm_gb300 import build as native
        native.build()
        print(json.dumps({"shear": run_shear(args)}))
        return 0
    if args.serve_only:
        from gpu_dsm_gb300 import build as native
        native.build()
        sv = run_serve(args)
        sv.pop("_samples", None)  # G(t) arrays kept for the CPU leg's FP64 check
        print(json.dumps({"serve": sv}))
        return 0
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
