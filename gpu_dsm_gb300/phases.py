"""Where the step kernel's time goes: per-phase SM clock cycles per kMC event,
and a latency probe of the operations on the event path (sm_103a).

    python -m gpu_dsm_gb300.phases [--cases load,warp,single] [--probe]

Builds ``libgpudsm_phases.so`` (the library compiled with -DDSM_PHASE_CLOCKS:
the step kernel's event loop reads the SM clock at each phase boundary and
sums the cycles per phase over chains) and runs the equilibrium melt of the
headline workload's parameters (N_K = 200, beta = 1, G(t) with p = 64, m = 8):

  load    16384 chains, the library's default schedule (32 chain tiles per
          SM), one 5 tau_K window after three warm-up windows
  warp    304 chains, one warp (two 16-lane tiles) per SM, 200 tau_K
  single  one chain on the whole GPU (16 and 32 lanes), 5000 tau_K: the
          latency of a chain that shares nothing

Phase cycles are those of each chain's own tile, so in a warp of two tiles a
phase also holds the time the warp spent on the other tile's diverging path.
A phase ends when its last instruction issues, so the latency of a result is
counted in the phase that first waits for it.  The clock reads add a few
percent: timings of the normal library are the bench's.

--probe compiles csrc/latency_probe.cu and prints cycles per operation of the
event path's building blocks (dependent chains on one warp).

Each case prints one JSON line."""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import subprocess
import sys

from . import build as native

NAMES = ["checks and correlator samples", "chain-end rates, rate passes, prefix rebuild", "dt",
         "Philox, pick, chunk walk", "classification", "apply: slide", "apply: destruction", "apply: creation",
         "pair-rate update, prefix patch", "event hash, counters", "chain load, first rate pass", "chain store"]
TYPES = ["slide", "destruction", "creation"]


def _load():
    lib_path = native.build(phases=True)
    os.environ["GPU_DSM_LIB"] = str(lib_path)
    from . import api
    if api._LIB is not None and getattr(api._LIB, "_name", "") != str(lib_path):
        raise RuntimeError("the normal library is already loaded in this process; run phases in a fresh process")
    lib = api.load_library()
    lib.dsm_phase_read.argtypes = [C.c_void_p]
    lib.dsm_phase_read.restype = C.c_int
    lib.dsm_phase_clear.restype = C.c_int
    return api, lib


def run_case(api, lib, tag: str, n: int, window: float, warm: int, **kw) -> dict:
    e = api.Ensemble(beta=1.0, nk=200, n_chains=n, eq_type=1, sync_dt=1.0, t_end=1.0e7, seed=1, corr_p=64, corr_m=8,
                     **kw)
    try:
        e.init_equilibrium()
        t = 0.0
        for _ in range(warm):
            t += window
            e.advance(t)
        if lib.dsm_phase_clear() != 0:
            raise RuntimeError("dsm_phase_clear")
        t += window
        ev = e.advance(t)
        lw = e.last_window()
        buf = (C.c_ulonglong * 32)()
        if lib.dsm_phase_read(buf) != 0:
            raise RuntimeError("dsm_phase_read")
    finally:
        e.close()
    g = list(buf)
    evp = max(1, g[20])
    per = {NAMES[k]: g[k] / evp for k in range(12)}
    loop = sum(g[k] for k in range(10)) / evp
    return {"case": tag, "chains": n, "events": ev, "kernel_ms": lw["kernel_ms"],
            "events_per_s_instrumented": ev / (lw["kernel_ms"] / 1e3), "cycles_per_event": per,
            "event_loop_cycles_per_event": loop,
            "event_share": {TYPES[i]: g[16 + i] / evp for i in range(3)},
            "apply_cycles_per_event_of_type": {TYPES[i]: g[5 + i] / max(1, g[16 + i]) for i in range(3)}}


def run_probe() -> dict:
    src = native.CSRC / "latency_probe.cu"
    exe = native.BUILD_PHASES / "latency_probe"
    native.BUILD_PHASES.mkdir(exist_ok=True)
    subprocess.run([native.nvcc(), *native.ARCH, "-O3", "-fmad=false", "-o", str(exe), str(src)], check=True)
    r = subprocess.run([str(exe)], check=True, capture_output=True, text=True)
    return {"case": "latency_probe", "cycles_per_op": json.loads(r.stdout.strip().splitlines()[-1])}


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--cases", default="load,warp,single")
    ap.add_argument("--probe", action="store_true")
    a = ap.parse_args(argv)
    if a.probe:
        print(json.dumps(run_probe()), flush=True)
    cases = [c for c in a.cases.split(",") if c]
    if not cases:
        return 0
    api, lib = _load()
    for c in cases:
        if c == "load":
            out = [run_case(api, lib, "load", 16384, 5.0, 3)]
        elif c == "warp":
            out = [run_case(api, lib, "one_warp_per_sm", 304, 200.0, 1, lanes_per_chain=16, warps_per_block=1)]
        elif c == "single":
            out = [run_case(api, lib, "single_chain_16_lanes", 1, 5000.0, 1, lanes_per_chain=16, warps_per_block=1),
                   run_case(api, lib, "single_chain_32_lanes", 1, 5000.0, 1, lanes_per_chain=32, warps_per_block=1)]
        else:
            raise SystemExit(f"unknown case {c}")
        for o in out:
            print(json.dumps(o), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
