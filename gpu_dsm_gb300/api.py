"""ctypes mirror of include/dsm.h.

``Ensemble`` plays the role of the reference's ensemble / call-block API
(common/ensemble.h:54-77, common/ensemble_call_block.h:55-75) for one
ensemble on one GPU: equilibrium initialisation, conformation transfer in the
reference layout, time evolution to a target time, flow stress and G(t).
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path
from typing import Optional, Sequence

import numpy as np

_PKG = Path(__file__).resolve().parent
_LIB: Optional[C.CDLL] = None

DSM_OK = 0
DSM_PENDING = 1
DSM_ABORTED = -1


class DSMError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"dsm error {code}: {msg}")
        self.code = code


class DsmParams(C.Structure):
    _fields_ = [
        ("beta", C.c_float),
        ("nk", C.c_int32),
        ("n_chains", C.c_int32),
        ("kappa", C.c_float * 9),
        ("cd_flag", C.c_int32),
        ("pd_flag", C.c_int32),
        ("eq_type", C.c_int32),
        ("sync_dt", C.c_double),
        ("t_end", C.c_double),
        ("seed", C.c_uint64),
        ("device", C.c_int32),
        ("z_max", C.c_int32),
        ("corr_p", C.c_int32),
        ("corr_m", C.c_int32),
        ("corr_levels", C.c_int32),
        ("stream", C.c_uint32),
        ("nk_chain", C.c_void_p),
        ("warps_per_block", C.c_int32),
        ("s0", C.c_int32),
        ("lanes_per_chain", C.c_int32),
        ("stream_priority", C.c_int32),
        ("gex_a", C.c_float),
        ("gex_b", C.c_float),
        ("gex_mp", C.c_float),
        ("gex_mk", C.c_float),
        ("chain_offset", C.c_uint32),
        ("pad2_", C.c_int32),
    ]


class ChainHead(C.Structure):
    _fields_ = [("Z", C.c_int32), ("time", C.c_float), ("dummy", C.c_float), ("stall_flag", C.c_int32)]


class StressPlus(C.Structure):
    _fields_ = [(n, C.c_float) for n in ("xx", "yy", "zz", "xy", "yz", "zx", "Lpp", "Z")]

    def as_array(self) -> np.ndarray:
        return np.array([getattr(self, n) for n, _ in self._fields_], dtype=np.float64)


class ServeTotals(C.Structure):
    _fields_ = [("events", C.c_uint64), ("busy_s", C.c_double), ("ticks", C.c_uint64), ("completed", C.c_uint64),
                ("peak_bytes", C.c_uint64), ("peak_active", C.c_int32), ("pad_", C.c_int32),
                ("setup_s", C.c_double), ("finish_s", C.c_double)]


HEAD_DTYPE = np.dtype([("Z", np.int32), ("time", np.float32), ("dummy", np.float32), ("stall_flag", np.int32)])


def lib_path() -> Path:
    """libgpudsm.so next to this module; GPU_DSM_LIB overrides the path."""
    env = os.environ.get("GPU_DSM_LIB")
    return Path(env) if env else _PKG / "libgpudsm.so"


def load_library() -> C.CDLL:
    """Load libgpudsm.so (built in-tree by gpu_dsm_gb300/build.py).  Raises if absent."""
    global _LIB
    if _LIB is not None:
        return _LIB
    p = lib_path()
    if not p.exists():
        raise DSMError(-6, f"native library {p} is missing: run gpu_dsm_gb300/build.py (nvcc, sm_103a)")
    lib = C.CDLL(str(p))
    vp, i32, i64, u64 = C.c_void_p, C.c_int32, C.c_int64, C.c_uint64
    lib.dsm_create.argtypes = [C.POINTER(DsmParams), C.POINTER(vp)]
    lib.dsm_create.restype = C.c_int
    lib.dsm_destroy.argtypes = [vp]
    lib.dsm_destroy.restype = None
    lib.dsm_last_error.argtypes = [vp]
    lib.dsm_last_error.restype = C.c_char_p
    lib.dsm_init_equilibrium.argtypes = [vp]
    lib.dsm_set_chains.argtypes = [vp, vp, vp, vp]
    lib.dsm_get_chains.argtypes = [vp, vp, vp, vp]
    lib.dsm_get_ext.argtypes = [vp, vp, vp, vp, vp, vp, vp]
    lib.dsm_set_ext.argtypes = [vp, vp, vp, vp, vp, vp]
    lib.dsm_advance.argtypes = [vp, C.c_double, i64, vp, vp]
    lib.dsm_stress.argtypes = [vp, C.POINTER(StressPlus), C.POINTER(i32)]
    lib.dsm_gt.argtypes = [vp, vp, vp, C.POINTER(i32)]
    lib.dsm_gt_raw.argtypes = [vp, vp, vp]
    lib.dsm_corr_shape.argtypes = [vp, C.POINTER(i32), C.POINTER(i32), C.POINTER(i32)]
    lib.dsm_last_window.argtypes = [vp, C.POINTER(C.c_float), C.POINTER(u64), C.POINTER(i32), C.POINTER(i32)]
    lib.dsm_last_window.restype = C.c_int
    lib.dsm_advance_batch.argtypes = [vp, i32, vp, vp, vp]
    lib.dsm_advance_batch.restype = C.c_int
    lib.dsm_save_file.argtypes = [vp, C.c_char_p]
    lib.dsm_load_file.argtypes = [vp, C.c_char_p]
    lib.dsm_checkpoint_save.argtypes = [vp, C.c_char_p]
    lib.dsm_checkpoint_load.argtypes = [vp, C.c_char_p]
    lib.dsm_advance_series.argtypes = [vp, C.c_double, i32, vp, vp, C.POINTER(u64)]
    lib.dsm_advance_series.restype = C.c_int
    lib.dsm_advance_start.argtypes = [vp, C.c_double, i64]
    lib.dsm_series_start.argtypes = [vp, vp, i32]
    lib.dsm_poll.argtypes = [vp, C.POINTER(u64), vp, C.POINTER(i32)]
    lib.dsm_abort.argtypes = [vp]
    for fn in ("dsm_advance_start", "dsm_series_start", "dsm_poll", "dsm_abort"):
        getattr(lib, fn).restype = C.c_int
    lib.dsm_autotune.argtypes = [vp, C.c_double, vp, C.POINTER(C.c_float)]
    lib.dsm_autotune.restype = C.c_int
    lib.dsm_zn_hist.argtypes = [vp, vp, i32, vp, i32]
    lib.dsm_zn_hist.restype = C.c_int
    lib.dsm_q_sorted.argtypes = [vp, vp, C.POINTER(i64)]
    lib.dsm_q_sorted.restype = C.c_int
    lib.dsm_get_r1.argtypes = [vp, vp]
    lib.dsm_get_r1.restype = C.c_int
    lib.dsm_window_stats.argtypes = [vp, C.POINTER(u64), C.POINTER(u64), C.POINTER(u64)]
    lib.dsm_window_stats.restype = C.c_int
    lib.dsm_set_schedule.argtypes = [vp, i32, i32, i32, C.c_float]
    lib.dsm_set_schedule.restype = C.c_int
    lib.dsm_get_schedule.argtypes = [vp, C.POINTER(i32), vp]
    lib.dsm_get_schedule.restype = C.c_int
    lib.dsm_set_class_form.argtypes = [vp, i32]
    lib.dsm_set_class_form.restype = C.c_int
    lib.dsm_get_class_form.argtypes = [vp, C.POINTER(i32)]
    lib.dsm_get_class_form.restype = C.c_int
    lib.dsm_gex_table.argtypes = [C.c_float] * 4 + [C.c_double, vp, C.POINTER(i32), vp, C.POINTER(i32), vp]
    lib.dsm_gex_table.restype = C.c_int
    lib.dsm_pcd.argtypes = [C.c_double, i32, vp]
    lib.dsm_pcd.restype = C.c_int
    lib.dsm_serve_open.argtypes = [i32, u64, i32, C.c_double, C.POINTER(vp)]
    lib.dsm_serve_submit.argtypes = [vp, C.POINTER(DsmParams), C.POINTER(u64)]
    lib.dsm_serve_status.argtypes = [vp, u64, C.POINTER(i32), C.POINTER(C.c_double), C.POINTER(C.c_double),
                                     C.POINTER(u64)]
    lib.dsm_serve_wait_all.argtypes = [vp, C.c_double]
    lib.dsm_serve_result_gt.argtypes = [vp, u64, vp, vp, C.POINTER(i32)]
    lib.dsm_serve_result_stress.argtypes = [vp, u64, vp, vp, C.POINTER(i32)]
    lib.dsm_serve_stats.argtypes = [vp, C.POINTER(ServeTotals)]
    lib.dsm_serve_set_policy.argtypes = [vp, i32]
    lib.dsm_serve_set_policy.restype = C.c_int
    lib.dsm_serve_tune.argtypes = [vp, C.c_double, C.c_double]
    lib.dsm_serve_tune.restype = C.c_int
    lib.dsm_serve_error.argtypes = [vp, u64]
    lib.dsm_serve_error.restype = C.c_char_p
    lib.dsm_serve_close.argtypes = [vp]
    lib.dsm_serve_close.restype = None
    for fn in ("dsm_init_equilibrium", "dsm_set_chains", "dsm_get_chains", "dsm_get_ext", "dsm_set_ext",
               "dsm_advance", "dsm_stress", "dsm_gt", "dsm_gt_raw", "dsm_corr_shape", "dsm_save_file",
               "dsm_load_file", "dsm_serve_open", "dsm_serve_submit", "dsm_serve_status", "dsm_serve_wait_all",
               "dsm_serve_result_gt", "dsm_serve_result_stress", "dsm_serve_stats"):
        getattr(lib, fn).restype = C.c_int
    _LIB = lib
    return lib


def _ptr(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def pcd(beta: float, nk: int) -> dict:
    """p_cd(beta, N_K) constants (common/pcd_tau.h:26-66): alpha, tau_0, tau_max, tau_d, g, normdt."""
    out = np.zeros(6, np.float64)
    rc = load_library().dsm_pcd(beta, nk, _ptr(out))
    if rc != DSM_OK:
        raise DSMError(rc, "dsm_pcd")
    return dict(zip(("alpha", "tau_0", "tau_max", "tau_d", "g", "normdt"), out.tolist()))


def gex_tables(a: float, b: float, mp: float, mk: float, beta: float) -> dict:
    """GEX background tables the library builds for pd_flag = 1 (dsm_gex_table):
    M/mp and CD-weighted inverse tables, their steps, mp/Mk and the CD creation
    prefactor (common/gamma.cpp:174-263, common/ensemble.cu:137-146)."""
    lib = load_library()
    cap = 4_000_000
    m, md = np.zeros(cap, np.float32), np.zeros(cap, np.float32)
    n, nd = C.c_int32(cap), C.c_int32(cap)
    info = np.zeros(3, np.float64)
    rc = lib.dsm_gex_table(a, b, mp, mk, beta, _ptr(m), C.byref(n), _ptr(md), C.byref(nd), _ptr(info))
    if rc != DSM_OK:
        raise DSMError(rc, "dsm_gex_table")
    return {"M": m[: n.value].copy(), "Md": md[: nd.value].copy(), "step": float(info[0]),
            "step_d": float(info[1]), "scale": float(np.float32(mp) / np.float32(mk)), "prefact": float(info[2])}


def make_params(*, beta: float = 1.0, nk: int, n_chains: int, kappa: Sequence[float] = (0.0,) * 9,
                cd_flag: int = 1, eq_type: int = 0, sync_dt: float = 1.0, t_end: float = 0.0, seed: int = 1,
                device: int = 0, z_max: int = 0, corr_p: int = 0, corr_m: int = 0, corr_levels: int = 0,
                stream: int = 0, warps_per_block: int = 0, s0: int = 0, lanes_per_chain: int = 0,
                gex: Optional[Sequence[float]] = None, chain_offset: int = 0) -> DsmParams:
    """dsm_params of an ensemble (input.dat fields, common/main_cuda.cu:55-68).
    gex = (a, b, mp, Mk) of polydisp.dat switches on the GEX background (pd_flag 1)."""
    p = DsmParams()
    p.beta = beta
    p.nk = nk
    p.n_chains = n_chains
    for i, k in enumerate(kappa):
        p.kappa[i] = k
    p.cd_flag = cd_flag
    p.pd_flag = 0 if gex is None else 1
    if gex is not None:
        p.gex_a, p.gex_b, p.gex_mp, p.gex_mk = (float(v) for v in gex)
    p.eq_type = eq_type
    p.sync_dt = sync_dt
    p.t_end = t_end
    p.seed = seed
    p.device = device
    p.z_max = z_max
    p.corr_p = corr_p
    p.corr_m = corr_m
    p.corr_levels = corr_levels
    p.stream = stream
    p.nk_chain = None
    p.warps_per_block = warps_per_block
    p.s0 = s0
    p.lanes_per_chain = lanes_per_chain
    p.chain_offset = chain_offset
    return p


class Ensemble:
    """One DSM ensemble resident on one GPU.

    Parameters mirror input.dat (common/main_cuda.cu:55-68): beta, nk, n_chains,
    kappa (9, row-major), cd_flag, eq_type (1 = G(t)), sync_dt, t_end; plus
    seed (job_ID), z_max (strand capacity, default nk), correlator p/m/levels,
    stream (ensemble id for the RNG), nk_chain (polydisperse per-chain N_K).
    """

    def __init__(self, *, beta: float = 1.0, nk: int, n_chains: int, kappa: Sequence[float] = (0.0,) * 9,
                 cd_flag: int = 1, eq_type: int = 0, sync_dt: float = 1.0, t_end: float = 0.0, seed: int = 1,
                 device: int = 0, z_max: int = 0, corr_p: int = 0, corr_m: int = 0, corr_levels: int = 0,
                 stream: int = 0, nk_chain: Optional[np.ndarray] = None, warps_per_block: int = 0, s0: int = 0,
                 lanes_per_chain: int = 0, gex: Optional[Sequence[float]] = None, chain_offset: int = 0):
        self._lib = load_library()
        self._nk_chain = None if nk_chain is None else np.ascontiguousarray(nk_chain, dtype=np.int32)
        p = make_params(beta=beta, nk=nk, n_chains=n_chains, kappa=kappa, cd_flag=cd_flag, eq_type=eq_type,
                        sync_dt=sync_dt, t_end=t_end, seed=seed, device=device, z_max=z_max, corr_p=corr_p,
                        corr_m=corr_m, corr_levels=corr_levels, stream=stream, warps_per_block=warps_per_block,
                        s0=s0, lanes_per_chain=lanes_per_chain, gex=gex, chain_offset=chain_offset)
        p.nk_chain = None if self._nk_chain is None else self._nk_chain.ctypes.data
        self.params = p
        self.n_chains = n_chains
        self.z_max = z_max if z_max > 0 else nk
        self.nk = nk
        h = C.c_void_p()
        rc = self._lib.dsm_create(C.byref(p), C.byref(h))
        self._h = h
        if rc != DSM_OK:
            msg = self._lib.dsm_last_error(h).decode() if h else ""
            self.close()
            raise DSMError(rc, msg)

    # ------------------------------------------------------------- plumbing
    def _check(self, rc: int) -> int:
        if rc not in (DSM_OK,):
            raise DSMError(rc, self._lib.dsm_last_error(self._h).decode())
        return rc

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.dsm_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ------------------------------------------------------------- state
    def init_equilibrium(self) -> None:
        self._check(self._lib.dsm_init_equilibrium(self._h))

    def get_chains(self, out=None):
        """Returns (heads structured array, QN float32 [n, z_max, 4], tau float32 [n, z_max]),
        written into ``out`` = (heads, qn, tau) when given (e.g. views of pinned host buffers)."""
        n, cap = self.n_chains, self.z_max
        if out is not None:
            heads, qn, tau = out
            assert heads.dtype == HEAD_DTYPE and heads.shape == (n,) and heads.flags.c_contiguous
            assert qn.dtype == np.float32 and qn.shape == (n, cap, 4) and qn.flags.c_contiguous
            assert tau.dtype == np.float32 and tau.shape == (n, cap) and tau.flags.c_contiguous
        else:
            heads = np.zeros(n, dtype=HEAD_DTYPE)
            qn = np.zeros((n, cap, 4), dtype=np.float32)
            tau = np.zeros((n, cap), dtype=np.float32)
        self._check(self._lib.dsm_get_chains(self._h, _ptr(heads), _ptr(qn), _ptr(tau)))
        return heads, qn, tau

    def set_chains(self, heads: np.ndarray, qn: np.ndarray, tau: np.ndarray) -> None:
        heads = np.ascontiguousarray(heads, dtype=HEAD_DTYPE)
        qn = np.ascontiguousarray(qn, dtype=np.float32)
        tau = np.ascontiguousarray(tau, dtype=np.float32)
        assert qn.shape == (self.n_chains, self.z_max, 4) and tau.shape == (self.n_chains, self.z_max)
        self._check(self._lib.dsm_set_chains(self._h, _ptr(heads), _ptr(qn), _ptr(tau)))

    def get_ext(self) -> dict:
        n = self.n_chains
        out = {"T": np.zeros(n, np.int64), "step": np.zeros(n, np.uint64), "dt_prev": np.zeros(n, np.float32),
               "stall": np.zeros(n, np.int32), "S": np.zeros(n, np.int32), "hash": np.zeros(n, np.uint64)}
        self._check(self._lib.dsm_get_ext(self._h, _ptr(out["T"]), _ptr(out["step"]), _ptr(out["dt_prev"]),
                                          _ptr(out["stall"]), _ptr(out["S"]), _ptr(out["hash"])))
        return out

    def set_ext(self, T=None, step=None, dt_prev=None, stall=None, S=None) -> None:
        conv = lambda a, t: None if a is None else np.ascontiguousarray(a, dtype=t)
        T, step, dt_prev, stall, S = (conv(T, np.int64), conv(step, np.uint64), conv(dt_prev, np.float32),
                                      conv(stall, np.int32), conv(S, np.int32))
        self._check(self._lib.dsm_set_ext(self._h, _ptr(T), _ptr(step), _ptr(dt_prev), _ptr(stall), _ptr(S)))

    # ------------------------------------------------------------- evolution
    def advance(self, t_end: float, step_limit: int = -1, abort: Optional[np.ndarray] = None) -> int:
        """Run all chains to time t_end (or step_limit events each).  Returns the events done.
        Returns -1 if aborted through ``abort`` (an int32 numpy scalar array set non-zero)."""
        ev = C.c_uint64(0)
        rc = self._lib.dsm_advance(self._h, float(t_end), int(step_limit), _ptr(abort), C.byref(ev))
        if rc == DSM_ABORTED:
            return -1
        self._check(rc)
        return int(ev.value)

    def advance_series(self, dt: float, n: int, abort: Optional[np.ndarray] = None):
        """n windows of dt tau_K as one CUDA graph replay (dsm_advance_series).
        Returns (kMC events, stress after each window as an (n, 8) array for
        flow ensembles, else None)."""
        ev = C.c_uint64()
        out = (StressPlus * n)() if self.params.kappa[:] != [0.0] * 9 and any(self.params.kappa[:]) else None
        self._check(self._lib.dsm_advance_series(self._h, dt, n, _ptr(abort),
                                                 None if out is None else C.cast(out, C.c_void_p), C.byref(ev)))
        st = None if out is None else np.array([out[i].as_array() for i in range(n)], np.float32)
        return ev.value, st

    # ------------------------------------------------------- asynchronous form
    def advance_start(self, t_end: float, step_limit: int = -1) -> None:
        """Enqueue a window on the ensemble's own stream and return (dsm_advance_start)."""
        self._check(self._lib.dsm_advance_start(self._h, t_end, step_limit))
        self._pending_n = 1

    def series_start(self, t_ends) -> None:
        """Enqueue windows ending at t_ends as one graph replay (dsm_series_start)."""
        te = np.ascontiguousarray(t_ends, dtype=np.float64)
        self._check(self._lib.dsm_series_start(self._h, _ptr(te), len(te)))
        self._pending_n = len(te)

    def poll(self):
        """None while running; then (events, stress (n, 8) or None)."""
        ev, nout = C.c_uint64(), C.c_int32()
        n = max(1, getattr(self, "_pending_n", 1))
        out = (StressPlus * n)()
        rc = self._lib.dsm_poll(self._h, C.byref(ev), C.cast(out, C.c_void_p), C.byref(nout))
        if rc == DSM_PENDING:
            return None
        self._check(rc)
        st = np.array([out[i].as_array() for i in range(nout.value)], np.float32) if nout.value else None
        return ev.value, st

    def last_window(self) -> dict:
        """Step-kernel device time (ms, CUDA events on its stream), events and launch shape of the
        last advance()."""
        ms, ev, grid, bps = C.c_float(), C.c_uint64(), C.c_int32(), C.c_int32()
        self._check(self._lib.dsm_last_window(self._h, C.byref(ms), C.byref(ev), C.byref(grid), C.byref(bps)))
        return {"kernel_ms": float(ms.value), "events": int(ev.value), "grid": int(grid.value),
                "blocks_per_sm": int(bps.value)}

    def stress(self):
        s = StressPlus()
        cnt = C.c_int32(0)
        self._check(self._lib.dsm_stress(self._h, C.byref(s), C.byref(cnt)))
        return s.as_array(), int(cnt.value)

    def corr_shape(self):
        L, p, m = C.c_int32(), C.c_int32(), C.c_int32()
        self._check(self._lib.dsm_corr_shape(self._h, C.byref(L), C.byref(p), C.byref(m)))
        return L.value, p.value, m.value

    def gt_raw(self):
        L, p, _ = self.corr_shape()
        g = np.zeros(L * p, np.float64)
        c = np.zeros(L * p, np.int64)
        self._check(self._lib.dsm_gt_raw(self._h, _ptr(g), _ptr(c)))
        return g.reshape(L, p), c.reshape(L, p)

    def gt(self):
        n = C.c_int32(8192)
        t = np.zeros(8192, np.float32)
        g = np.zeros(8192, np.float32)
        self._check(self._lib.dsm_gt(self._h, _ptr(t), _ptr(g), C.byref(n)))
        return t[: n.value].copy(), g[: n.value].copy()

    def autotune(self, window: float) -> dict:
        """Pick the fastest launch schedule: one real window of ``window`` tau_K
        per candidate (the ensemble advances); returns the choice."""
        best = np.zeros(4, np.int32)
        ms = C.c_float()
        self._check(self._lib.dsm_autotune(self._h, window, _ptr(best), C.byref(ms)))
        return {"small_slot": int(best[0]), "large_grid": int(best[1]), "lanes": int(best[2]),
                "candidates": int(best[3]), "kernel_ms": ms.value}

    def distributions(self):
        """Device-computed statistics of the -distr files: (Z histogram over
        chains, N histogram over strands, sorted |Q| of the internal strands)."""
        nb = self.z_max + 2
        hz = np.zeros(nb, np.uint64)
        hn = np.zeros(max(nb, self.nk + 2), np.uint64)
        self._check(self._lib.dsm_zn_hist(self._h, _ptr(hz), nb, _ptr(hn), len(hn)))
        n = C.c_int64(0)
        self._check(self._lib.dsm_q_sorted(self._h, None, C.byref(n)))
        q = np.zeros(max(1, n.value), np.float32)
        self._check(self._lib.dsm_q_sorted(self._h, _ptr(q), C.byref(n)))
        return hz, hn, q[: n.value]

    def r1(self) -> np.ndarray:
        """MSD mode (eq_type=2): first-entanglement position of every chain, (n, 3)."""
        out = np.zeros((self.n_chains, 3), np.float32)
        self._check(self._lib.dsm_get_r1(self._h, _ptr(out)))
        return out

    def window_stats(self) -> dict:
        """Counters of the last window: events, chains done in their first slot, chains deferred."""
        a, b, c = C.c_uint64(), C.c_uint64(), C.c_uint64()
        self._check(self._lib.dsm_window_stats(self._h, C.byref(a), C.byref(b), C.byref(c)))
        return {"events": a.value, "chains_done": b.value, "deferred": c.value}

    def set_schedule(self, small_slot: int = 0, large_grid: int = 0, lanes: int = 0, z_margin_sd: float = 0.0) -> None:
        """Size-class launch schedule of a polydisperse ensemble (dsm_set_schedule)."""
        self._check(self._lib.dsm_set_schedule(self._h, small_slot, large_grid, lanes, z_margin_sd))

    def set_class_form(self, form: int) -> None:
        """0: size classes as concurrent launches; 1: large, middle and small
        classes in one carved launch (dsm_set_class_form)."""
        self._check(self._lib.dsm_set_class_form(self._h, form))

    def class_form(self) -> int:
        f = C.c_int32()
        self._check(self._lib.dsm_get_class_form(self._h, C.byref(f)))
        return f.value

    def schedule(self) -> list:
        """[{slot, warps_per_block, lanes, grid, chains}, ...]; empty for one launch over all chains."""
        n = C.c_int32()
        info = np.zeros(25, np.int32)  # DSM_SCHEDULE_INFO
        self._check(self._lib.dsm_get_schedule(self._h, C.byref(n), _ptr(info)))
        keys = ("slot", "warps_per_block", "lanes", "grid", "chains")
        m = n.value + 1 if n.value else 0
        return [dict(zip(keys, info[5 * i:5 * i + 5].tolist())) for i in range(m)]

    def save(self, path: str) -> None:
        self._check(self._lib.dsm_save_file(self._h, os.fsencode(path)))

    def load(self, path: str) -> None:
        self._check(self._lib.dsm_load_file(self._h, os.fsencode(path)))

    def checkpoint(self, path: str) -> None:
        """Full-state checkpoint for an exact resume (dsm_checkpoint_save)."""
        self._check(self._lib.dsm_checkpoint_save(self._h, os.fsencode(path)))

    def restore(self, path: str) -> None:
        """Restore a full-state checkpoint written by an ensemble of the same shape and
        random streams (dsm_checkpoint_load); the ensemble is unchanged on failure."""
        self._check(self._lib.dsm_checkpoint_load(self._h, os.fsencode(path)))


def advance_batch(ensembles, t_end, step_limit=None):
    """Advance several Ensemble objects (same GPU) in one persistent launch per kind.
    Returns the kMC events of each ensemble."""
    lib = load_library()
    n = len(ensembles)
    hs = (C.c_void_p * n)(*[e._h.value for e in ensembles])
    te = np.ascontiguousarray(np.broadcast_to(np.asarray(t_end, np.float64), (n,)))
    sl = None if step_limit is None else np.ascontiguousarray(np.broadcast_to(np.asarray(step_limit, np.int64), (n,)))
    ev = np.zeros(n, np.uint64)
    rc = lib.dsm_advance_batch(C.cast(hs, C.c_void_p), n, _ptr(te), _ptr(sl), _ptr(ev))
    if rc != DSM_OK:
        raise DSMError(rc, lib.dsm_last_error(ensembles[0]._h).decode())
    return ev


REQ_QUEUED, REQ_ACTIVE, REQ_DONE, REQ_FAILED = 0, 1, 2, 3


class Server:
    """Continuous-batching serving loop on one GPU (dsm_serve_* of the C ABI).

    Requests (keyword arguments of ``make_params``) are admitted while their
    ensembles fit in ``hbm_budget`` bytes of device memory, stay resident and
    run concurrently, each on its own stream in chunks of about ``chunk_s``
    seconds.  ``max_active=1, chunk_s=-1`` is the plain form: one request at a
    time, one launch per request (equilibrium) or per output (flow).
    """

    POLICIES = {"fcfs": 0, "equal_pace": 1, "fcfs_strict": 2}

    def __init__(self, *, device: int = 0, hbm_budget: int = 0, max_active: int = 0, chunk_s: float = 0.0,
                 policy: str = "fcfs", overlap: float = 1.0, bypass: float = 0.2):
        self._lib = load_library()
        h = C.c_void_p()
        rc = self._lib.dsm_serve_open(device, hbm_budget, max_active, chunk_s, C.byref(h))
        if rc != DSM_OK:
            raise DSMError(rc, "dsm_serve_open")
        self._h = h
        rc = self._lib.dsm_serve_set_policy(h, self.POLICIES[policy])
        if rc == DSM_OK:
            rc = self._lib.dsm_serve_tune(h, overlap, bypass)
        if rc != DSM_OK:
            raise DSMError(rc, "dsm_serve_set_policy")
        self.device = device

    def submit(self, **kw) -> int:
        kw.setdefault("device", self.device)
        p = make_params(**kw)
        rid = C.c_uint64()
        rc = self._lib.dsm_serve_submit(self._h, C.byref(p), C.byref(rid))
        if rc != DSM_OK:
            raise DSMError(rc, "dsm_serve_submit")
        return rid.value

    def status(self, rid: int) -> dict:
        st, lat, q, ev = C.c_int32(), C.c_double(), C.c_double(), C.c_uint64()
        rc = self._lib.dsm_serve_status(self._h, rid, C.byref(st), C.byref(lat), C.byref(q), C.byref(ev))
        if rc != DSM_OK:
            raise DSMError(rc, "dsm_serve_status")
        d = {"state": st.value, "latency_s": lat.value, "queue_s": q.value, "events": ev.value}
        if st.value == REQ_FAILED:
            d["error"] = self._lib.dsm_serve_error(self._h, rid).decode()
        return d

    def wait_all(self, timeout_s: float = 3600.0) -> None:
        rc = self._lib.dsm_serve_wait_all(self._h, timeout_s)
        if rc != DSM_OK:
            raise DSMError(rc, "dsm_serve_wait_all")

    def result_gt(self, rid: int):
        n = C.c_int32(0)
        self._lib.dsm_serve_result_gt(self._h, rid, None, None, C.byref(n))
        t = np.zeros(max(n.value, 1), np.float32)
        g = np.zeros(max(n.value, 1), np.float32)
        rc = self._lib.dsm_serve_result_gt(self._h, rid, _ptr(t), _ptr(g), C.byref(n))
        if rc != DSM_OK:
            raise DSMError(rc, "dsm_serve_result_gt")
        return t[:n.value], g[:n.value]

    def result_stress(self, rid: int):
        n = C.c_int32(0)
        self._lib.dsm_serve_result_stress(self._h, rid, None, None, C.byref(n))
        t = np.zeros(max(n.value, 1), np.float64)
        s = (StressPlus * max(n.value, 1))()
        rc = self._lib.dsm_serve_result_stress(self._h, rid, _ptr(t), C.cast(s, C.c_void_p), C.byref(n))
        if rc != DSM_OK:
            raise DSMError(rc, "dsm_serve_result_stress")
        return t[:n.value], np.array([s[i].as_array() for i in range(n.value)], np.float32).reshape(n.value, -1)

    def stats(self) -> dict:
        t = ServeTotals()
        rc = self._lib.dsm_serve_stats(self._h, C.byref(t))
        if rc != DSM_OK:
            raise DSMError(rc, "dsm_serve_stats")
        d = {n: getattr(t, n) for n, _ in ServeTotals._fields_ if n != "pad_"}
        d["chunks"] = d.pop("ticks")
        return d

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.dsm_serve_close(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
