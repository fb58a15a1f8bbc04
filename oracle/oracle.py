"""ORACLE — test infrastructure only.

ctypes binding of ``oracle/liboracle.so`` (the CPU restatement of the
reference DSM kMC path, see dsm_oracle.cpp), of ``oracle/_ref/libdsmref.so``
(the reference's own host initialiser and p_cd, compiled from the reference
tree) and of ``oracle/_ref/libdsmrefstep.so`` (the reference's kMC kernels
compiled unchanged for the host, driven by ref_step.cpp).  The reference tree is
found at $GPU_DSM_REFERENCE (default /root/reference).  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline /
reference legs use this module, as the checker or the timed CPU restatement.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path
from typing import Optional

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "liboracle.so"
REFLIB = HERE / "_ref" / "libdsmref.so"
REFSTEPLIB = HERE / "_ref" / "libdsmrefstep.so"
REFSRC = Path(os.environ.get("GPU_DSM_REFERENCE", "/root/reference")) / "common"


class OrcParams(C.Structure):
    _fields_ = [
        ("beta", C.c_double), ("nk", C.c_int32), ("n_chains", C.c_int32), ("z_max", C.c_int32),
        ("cd_flag", C.c_int32), ("kappa", C.c_float * 9), ("mode", C.c_int32), ("stream", C.c_uint32),
        ("seed", C.c_uint64), ("corr_type", C.c_int32), ("corr_p", C.c_int32), ("corr_m", C.c_int32),
        ("corr_levels", C.c_int32), ("corr_dt", C.c_double), ("corr_nsamples", C.c_int64),
        ("nk_chain", C.c_void_p), ("s0", C.c_int32), ("gex", C.c_int32),
        ("gex_M", C.c_void_p), ("gex_Md", C.c_void_p), ("gex_n", C.c_int32), ("gex_nd", C.c_int32),
        ("gex_step", C.c_float), ("gex_step_d", C.c_float), ("gex_scale", C.c_float), ("pad2_", C.c_int32),
        ("gex_prefact", C.c_double), ("chain_offset", C.c_uint32), ("partner_n", C.c_int32),
        ("partner_nk", C.c_void_p),
    ]


def build(ref: bool = False) -> None:
    """make liboracle.so (and _ref/libdsmref.so when the reference tree exists)."""
    subprocess.run(["make", "-s", "-C", str(HERE), "liboracle.so"], check=True)
    if ref and REFSRC.exists():
        subprocess.run(["make", "-s", "-C", str(HERE), "ref", f"GPU_DSM_REFERENCE={REFSRC.parent}"], check=True)


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        L = C.CDLL(str(LIB))
        vp = C.c_void_p
        L.orc_create.argtypes = [C.POINTER(OrcParams)]
        L.orc_create.restype = vp
        L.orc_destroy.argtypes = [vp]
        L.orc_init_equilibrium.argtypes = [vp, C.c_int]
        L.orc_set_state.argtypes = [vp] + [vp] * 8
        L.orc_get_state.argtypes = [vp] + [vp] * 9
        L.orc_run.argtypes = [vp, C.c_double, C.c_int64, C.c_int]
        L.orc_run.restype = C.c_int64
        L.orc_stress.argtypes = [vp, vp, vp]
        L.orc_gt.argtypes = [vp, vp, vp]
        L.orc_pcd.argtypes = [C.c_double, C.c_double, vp, vp]
        L.orc_philox.argtypes = [vp, vp, vp]
        L.orc_split.argtypes = [C.c_uint64, C.c_uint64, C.c_int]
        L.orc_split.restype = C.c_int
        L.orc_math.argtypes = [C.c_int, vp, vp, vp, C.c_int]
        L.orc_tau_sample.argtypes = [C.c_double, C.c_double, C.c_int, C.c_int, vp, vp, C.c_int]
        L.orc_num_threads.restype = C.c_int
        L.orc_corr_series.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int64, vp, vp, vp]
        L.orc_get_r1.argtypes = [vp, vp]
        L.orc_get_ref.argtypes = [vp, vp, vp, vp]
        L.orc_ref_params.argtypes = [vp, vp, vp]
        L.orc_gt_chains.argtypes = [vp, vp]
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def corr_levels_for(t_end: float, dt: float, p: int, m: int) -> int:
    """common/main_cuda.cu:70"""
    import math
    return max(1, int(math.ceil(math.log(t_end / dt / p) / math.log(m)) + 1))


class Oracle:
    """One ensemble on the CPU.  mode 0 = FP32 mirror of the GPU arithmetic,
    mode 1 = FP64 literal transcription, mode 2 = the reference's own
    arithmetic (FP32 rates, running-sum scan, FP32 window clocks).  In mode 2
    ``run(t_end, step_limit)`` follows the reference's step loops: t_end is the
    absolute time to reach, step_limit an absolute event count."""

    def __init__(self, *, beta=1.0, nk, n_chains, z_max=0, cd_flag=1, kappa=(0.0,) * 9, mode=0, seed=1,
                 stream=0, corr=False, corr_p=64, corr_m=8, corr_levels=0, sync_dt=1.0, t_end=0.0,
                 nk_chain: Optional[np.ndarray] = None, s0=0, threads=0, msd=False, gex_tables=None,
                 chain_offset=0, partner_nk: Optional[np.ndarray] = None):
        L = lib()
        p = OrcParams()
        p.beta = float(np.float32(beta))
        p.nk = nk
        p.n_chains = n_chains
        p.z_max = z_max if z_max > 0 else nk
        p.cd_flag = cd_flag
        for i, k in enumerate(kappa):
            p.kappa[i] = k
        p.mode = mode
        p.stream = stream
        p.seed = seed
        flow = any(k != 0 for k in kappa)
        corr = corr or msd
        p.corr_type = (1 if msd else 0) if (corr and not flow) else -1
        p.corr_p, p.corr_m = corr_p, corr_m
        p.corr_levels = corr_levels if corr_levels > 0 else (corr_levels_for(t_end, sync_dt, corr_p, corr_m) if corr else 1)
        p.corr_dt = sync_dt
        import math
        p.corr_nsamples = int(math.ceil(t_end / sync_dt)) if corr else 0
        self._nk_chain = None if nk_chain is None else np.ascontiguousarray(nk_chain, dtype=np.int32)
        p.nk_chain = None if self._nk_chain is None else self._nk_chain.ctypes.data
        p.s0 = s0
        p.chain_offset = chain_offset
        # polydisperse slice of a larger ensemble: partners and the CD prefactor
        # come from the whole ensemble's per-chain N_K
        self._partner = None if partner_nk is None else np.ascontiguousarray(partner_nk, dtype=np.int32)
        if self._partner is not None:
            p.partner_nk = self._partner.ctypes.data
            p.partner_n = len(self._partner)
        if gex_tables is not None:
            # GEX background: inverse tables and prefactor as the product builds them
            self._gex_M = np.ascontiguousarray(gex_tables["M"], np.float32)
            self._gex_Md = np.ascontiguousarray(gex_tables["Md"], np.float32)
            p.gex = 1
            p.gex_M, p.gex_Md = self._gex_M.ctypes.data, self._gex_Md.ctypes.data
            p.gex_n, p.gex_nd = len(self._gex_M), len(self._gex_Md)
            p.gex_step, p.gex_step_d = gex_tables["step"], gex_tables["step_d"]
            p.gex_scale = gex_tables["scale"]
            p.gex_prefact = gex_tables["prefact"]
        self.p = p
        self.n = n_chains
        self.cap = p.z_max
        self.threads = threads if threads > 0 else L.orc_num_threads()
        self._h = L.orc_create(C.byref(p))

    def close(self):
        if self._h:
            lib().orc_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def init_equilibrium(self):
        lib().orc_init_equilibrium(self._h, self.threads)

    def set_state(self, Z, QN, tau, T=None, step=None, dt_prev=None, stall=None, S=None):
        a = lambda x, t: None if x is None else np.ascontiguousarray(x, dtype=t)
        Z, QN, tau = a(Z, np.int32), a(QN, np.float32), a(tau, np.float32)
        T, step, dt_prev, stall, S = a(T, np.int64), a(step, np.uint64), a(dt_prev, np.float32), a(stall, np.int32), a(S, np.int32)
        rc = lib().orc_set_state(self._h, _p(Z), _p(QN), _p(tau), _p(T), _p(step), _p(dt_prev), _p(stall), _p(S))
        assert rc == 0

    def get_state(self) -> dict:
        n, cap = self.n, self.cap
        d = {"Z": np.zeros(n, np.int32), "QN": np.zeros((n, cap, 4), np.float32), "tau": np.zeros((n, cap), np.float32),
             "T": np.zeros(n, np.int64), "step": np.zeros(n, np.uint64), "dt_prev": np.zeros(n, np.float32),
             "stall": np.zeros(n, np.int32), "S": np.zeros(n, np.int32), "hash": np.zeros(n, np.uint64)}
        lib().orc_get_state(self._h, _p(d["Z"]), _p(d["QN"]), _p(d["tau"]), _p(d["T"]), _p(d["step"]),
                            _p(d["dt_prev"]), _p(d["stall"]), _p(d["S"]), _p(d["hash"]))
        return d

    def run(self, t_end: float, step_limit: int = -1) -> int:
        return int(lib().orc_run(self._h, float(t_end), int(step_limit), self.threads))

    def stress(self):
        out = np.zeros(8, np.float64)
        cnt = np.zeros(1, np.int32)
        lib().orc_stress(self._h, _p(out), _p(cnt))
        return out, int(cnt[0])

    def r1(self):
        """MSD mode: first-entanglement position of every chain (n, 3)."""
        out = np.zeros((self.n, 3), np.float64)
        lib().orc_get_r1(self._h, _p(out))
        return out

    def gt_chains(self):
        """Per-chain correlator averages acc/count (n, levels, p)."""
        L, p = self.p.corr_levels, self.p.corr_p
        out = np.zeros(self.n * L * p, np.float64)
        assert lib().orc_gt_chains(self._h, _p(out)) == 0
        return out.reshape(self.n, L, p)

    def ref_clock(self):
        """Mode 2: FP32 time since the window start, sample counters, R1."""
        tf = np.zeros(self.n, np.float32)
        k = np.zeros(self.n, np.int32)
        r1 = np.zeros((self.n, 3), np.float32)
        assert lib().orc_get_ref(self._h, _p(tf), _p(k), _p(r1)) == 0
        return tf, k, r1

    def ref_params(self):
        """CD creation prefactor and lifetime-law constants (ref_tape.h order)."""
        pf = np.zeros(1, np.float32)
        law = np.zeros(9, np.float64)
        lib().orc_ref_params(self._h, _p(pf), _p(law))
        return float(pf[0]), law

    def gt_raw(self):
        L, p = self.p.corr_levels, self.p.corr_p
        g = np.zeros(L * p, np.float64)
        c = np.zeros(L * p, np.int64)
        lib().orc_gt(self._h, _p(g), _p(c))
        return g.reshape(L, p), c.reshape(L, p)


def pcd(beta: float, nk: float):
    out = np.zeros(12, np.float64)
    outf = np.zeros(9, np.float32)
    lib().orc_pcd(float(beta), float(nk), _p(out), _p(outf))
    return out, outf


def philox(ctr, key):
    c = np.asarray(ctr, np.uint32)
    k = np.asarray(key, np.uint32)
    o = np.zeros(4, np.uint32)
    lib().orc_philox(_p(c), _p(k), _p(o))
    return o


def math_f(which: int, x=None, w=None, n=None):
    x = None if x is None else np.ascontiguousarray(x, np.float32)
    w = None if w is None else np.ascontiguousarray(w, np.uint32)
    n = n if n is not None else (len(x) if x is not None else len(w))
    y = np.zeros(2 * n if which == 2 else n, np.float32)
    lib().orc_math(which, _p(x), _p(w), _p(y), n)
    return y


def tau_samples(beta, nk, kind, mode, u):
    u = np.ascontiguousarray(u, np.float32)
    out = np.zeros(len(u), np.float64)
    lib().orc_tau_sample(float(beta), float(nk), kind, mode, _p(u), _p(out), len(u))
    return out


# ---------------------------------------------------------------- compiled reference
_ref = None


def ref_lib() -> Optional[C.CDLL]:
    """The reference's own host code (only where the reference tree was available)."""
    global _ref
    if _ref is None:
        if not REFLIB.exists():
            if REFSRC.exists():
                build(ref=True)
            else:
                return None
        R = C.CDLL(str(REFLIB))
        R.ref_pcd.argtypes = [C.c_float, C.c_float, C.c_void_p]
        R.ref_chain_init.argtypes = [C.c_int, C.c_int, C.c_int, C.c_float, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
        R.ref_tau_samples.argtypes = [C.c_float, C.c_float, C.c_int, C.c_int, C.c_int, C.c_void_p]
        _ref = R
    return _ref


class RefParams(C.Structure):
    _fields_ = [
        ("n_chains", C.c_int32), ("nk", C.c_int32), ("z_max", C.c_int32), ("cd_flag", C.c_int32),
        ("beta", C.c_float), ("prefact", C.c_float), ("kappa", C.c_float * 9), ("eq", C.c_int32),
        ("corr_type", C.c_int32), ("corr_p", C.c_int32), ("corr_m", C.c_int32), ("corr_levels", C.c_int32),
        ("corr_res", C.c_int32), ("seed", C.c_uint64), ("stream", C.c_uint32), ("chain_offset", C.c_uint32),
        ("law", C.c_double * 9),
    ]


_refstep = None


def refstep_lib() -> Optional[C.CDLL]:
    """The reference's kMC kernels compiled for the host (None without the reference tree)."""
    global _refstep
    if _refstep is None:
        if not REFSTEPLIB.exists():
            if REFSRC.exists():
                build(ref=True)
            else:
                return None
        R = C.CDLL(str(REFSTEPLIB))
        vp = C.c_void_p
        R.ref_create.argtypes = [C.POINTER(RefParams)]
        R.ref_create.restype = vp
        R.ref_destroy.argtypes = [vp]
        R.ref_set_chains.argtypes = [vp] * 5
        R.ref_run.argtypes = [vp, C.c_double, C.c_int64]
        R.ref_get_chains.argtypes = [vp] * 9
        R.ref_stress.argtypes = [vp, vp, vp]
        R.ref_gt.argtypes = [vp, vp, vp, vp]
        _refstep = R
    return _refstep


class RefStep:
    """One call block of the reference's own kMC kernels (common/ensemble_kernel.cu,
    common/eq_ensemble_kernel.cu) run on the host by oracle/ref_step.cpp, fed
    the random stream of ``like`` (a mode-2 Oracle of the same ensemble).
    Equilibrium runs always carry the reference's correlator (sample interval
    ``corr_res``)."""

    def __init__(self, like: "Oracle", *, corr_res: int = 1):
        R = refstep_lib()
        assert R is not None, "reference tree not available"
        o = like.p
        pf, law = like.ref_params()
        p = RefParams()
        p.n_chains, p.nk, p.z_max, p.cd_flag = o.n_chains, o.nk, o.z_max, o.cd_flag
        p.beta, p.prefact = o.beta, pf
        for i in range(9):
            p.kappa[i] = o.kappa[i]
        flow = any(o.kappa[i] != 0.0 for i in range(9))
        p.eq = 0 if flow else 1
        p.corr_type = max(o.corr_type, 0)
        p.corr_p, p.corr_m, p.corr_levels = o.corr_p, o.corr_m, o.corr_levels
        p.corr_res = int(corr_res)
        p.seed, p.stream, p.chain_offset = o.seed, o.stream, o.chain_offset
        for i in range(9):
            p.law[i] = law[i]
        self.p = p
        self.n, self.cap = o.n_chains, o.z_max
        self._h = R.ref_create(C.byref(p))

    def close(self):
        if self._h:
            refstep_lib().ref_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_chains(self, Z, QN, tau, R1=None):
        a = lambda x, t: None if x is None else np.ascontiguousarray(x, dtype=t)
        Z, QN, tau, R1 = a(Z, np.int32), a(QN, np.float32), a(tau, np.float32), a(R1, np.float32)
        assert refstep_lib().ref_set_chains(self._h, _p(Z), _p(QN), _p(tau), _p(R1)) == 0

    def run(self, reach_time: float, event_limit: int = -1) -> int:
        """Returns 0, or the code of the first out-of-range surface access."""
        return int(refstep_lib().ref_run(self._h, float(reach_time), int(event_limit)))

    def get_state(self) -> dict:
        n, cap = self.n, self.cap
        d = {"Z": np.zeros(n, np.int32), "QN": np.zeros((n, cap, 4), np.float32), "tau": np.zeros((n, cap), np.float32),
             "time": np.zeros(n, np.float32), "stall": np.zeros(n, np.int32), "events": np.zeros(n, np.int64),
             "R1": np.zeros((n, 4), np.float32), "corr_time": np.zeros(n, np.int32)}
        refstep_lib().ref_get_chains(self._h, _p(d["Z"]), _p(d["QN"]), _p(d["tau"]), _p(d["time"]), _p(d["stall"]),
                                     _p(d["events"]), _p(d["R1"]), _p(d["corr_time"]))
        return d

    def stress(self):
        out = np.zeros(8, np.float64)
        cnt = np.zeros(1, np.int32)
        assert refstep_lib().ref_stress(self._h, _p(out), _p(cnt)) == 0
        return out, int(cnt[0])

    def gt(self):
        """corr_function_calc_kernel's ensemble sums (levels x p, float) and lags."""
        L, p = self.p.corr_levels, self.p.corr_p
        corr = np.zeros(L * p, np.float32)
        lag = np.zeros(L * p, np.float32)
        n0 = np.zeros(L * p, np.float32)
        refstep_lib().ref_gt(self._h, _p(corr), _p(lag), _p(n0))
        return corr.reshape(L, p), lag.reshape(L, p), n0.reshape(L, p)


def corr_series(series: np.ndarray, p: int, m: int, levels: int, kind: int = 0):
    """Run the oracle's multi-tau correlator (kind 0 products, 1 squared
    differences) on one series of 3-vectors."""
    x = np.ascontiguousarray(series, np.float64)
    acc = np.zeros(levels * p, np.float64)
    nins = np.zeros(levels, np.int64)
    lib().orc_corr_series(kind, p, m, levels, len(x), _p(x), _p(acc), _p(nins))
    return acc.reshape(levels, p), nins


def gt_error_vs_fp64(g_test: np.ndarray, fp64: "Oracle", prec: float = 0.02) -> dict:
    """Error of a G(t) (or MSD) estimate against the FP64 oracle run on the
    same chains and random stream.  Both inputs are correlator sums of shape
    (levels, p) normalised the same way; the FP64 ensemble's per-chain values
    give the statistical error sigma of its mean at every lag.

    rel_resolved: max |dG| / |G| over the lags the ensemble resolves to
        ``prec`` statistical precision (sigma < prec |G|);
    dev_sigma: max |dG| / sigma over all populated lags;
    rel_scale: max |dG| / |G(lag 0)|."""
    g_ref, cnt = fp64.gt_raw()
    per = fp64.gt_chains()
    n = per.shape[0]
    sig = per.std(axis=0, ddof=1) * n / np.sqrt(n)  # error of the sum over n chains
    m = cnt > 0
    d = np.abs(np.asarray(g_test, np.float64) - g_ref)
    res = m & (sig < prec * np.abs(g_ref))
    return {"rel_resolved": float((d[res] / np.abs(g_ref[res])).max()) if res.any() else None,
            "resolved_lags": int(res.sum()), "lags": int(m.sum()), "precision": prec,
            "dev_sigma": float((d[m] / np.maximum(sig[m], 1e-300)).max()),
            "rel_scale": float(d[m].max() / abs(g_ref[0, 0]))}


def gt_points_error_vs_fp64(g_points: np.ndarray, fp64: "Oracle", prec: float = 0.02) -> dict:
    """gt_error_vs_fp64 for a G(t) in the G.dat point order and normalisation
    (correlator.cu:146-187, ensemble.cu:318-335): level 0 lags 0..p-1, then
    lags p/m..p-1 of every further level, each sum / 3 / N_cha."""
    L, p, m = fp64.p.corr_levels, fp64.p.corr_p, fp64.p.corr_m
    n = fp64.n
    g_ref, cnt = fp64.gt_raw()
    per = fp64.gt_chains()

    def flat(a):
        rows = [a[..., 0, :]] + [a[..., k, p // m:] for k in range(1, L)]
        return np.concatenate(rows, axis=-1)

    npt = len(g_points)
    ref = flat(g_ref)[:npt] / 3.0 / n
    c = flat(cnt)[:npt]
    sig = flat(per).std(axis=0, ddof=1)[:npt] / np.sqrt(n) / 3.0
    d = np.abs(np.asarray(g_points, np.float64) - ref)
    m_ = c > 0
    res = m_ & (sig < prec * np.abs(ref))
    return {"rel_resolved": float((d[res] / np.abs(ref[res])).max()) if res.any() else None,
            "resolved_lags": int(res.sum()), "lags": int(m_.sum()), "precision": prec,
            "dev_sigma": float((d[m_] / np.maximum(sig[m_], 1e-300)).max()),
            "rel_scale": float(d[m_].max() / abs(ref[0]))}
