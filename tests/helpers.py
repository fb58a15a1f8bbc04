"""Shared helpers: run the same ensemble on the GPU (C ABI) and in the oracle."""
from __future__ import annotations

import numpy as np

STATE_KEYS = ("Z", "QN", "tau", "T", "step", "hash", "S", "stall")


def gpu_state(ens) -> dict:
    heads, qn, tau = ens.get_chains()
    ext = ens.get_ext()
    d = {"Z": heads["Z"].copy(), "QN": qn, "tau": tau}
    d.update({k: ext[k] for k in ("T", "step", "hash", "S", "stall", "dt_prev")})
    return d


def masked(d: dict) -> dict:
    """Zero everything beyond Z (strands) / Z-1 (entanglements)."""
    Z = d["Z"]
    cap = d["QN"].shape[1]
    idx = np.arange(cap)[None, :]
    qn = np.where((idx < Z[:, None])[..., None], d["QN"], 0).astype(np.float32)
    tau = np.where(idx < (Z[:, None] - 1), d["tau"], 0).astype(np.float32)
    out = dict(d)
    out["QN"], out["tau"] = qn, tau
    return out


def assert_bitexact(g: dict, o: dict, keys=STATE_KEYS, what=""):
    g, o = masked(g), masked(o)
    for k in keys:
        a, b = np.asarray(g[k]), np.asarray(o[k])
        if a.dtype.kind == "f":
            same = a.view(np.uint32 if a.dtype == np.float32 else np.uint64) == b.astype(a.dtype).view(
                np.uint32 if a.dtype == np.float32 else np.uint64)
        else:
            same = a == b.astype(a.dtype)
        if not np.all(same):
            bad = np.argwhere(~same)
            i = tuple(bad[0])
            raise AssertionError(f"{what}: {k} differs at {i} ({bad.shape[0]} entries): gpu={a[i]!r} oracle={b[i]!r}")


def pair(dsm, orc, *, nk, n, seed=1, beta=1.0, z_max=0, cd=1, kappa=(0.0,) * 9, corr=False, sync_dt=1.0,
         t_end=0.0, corr_p=16, corr_m=2, nk_chain=None, stream=0, lanes=0, msd=False):
    g = dsm.Ensemble(beta=beta, nk=nk, n_chains=n, z_max=z_max, cd_flag=cd, kappa=kappa,
                     eq_type=2 if msd else (1 if corr else 0), sync_dt=sync_dt, t_end=t_end, seed=seed,
                     corr_p=corr_p, corr_m=corr_m, nk_chain=nk_chain, stream=stream, lanes_per_chain=lanes)
    o = orc.Oracle(beta=beta, nk=nk, n_chains=n, z_max=z_max, cd_flag=cd, kappa=kappa, seed=seed,
                   corr=corr, sync_dt=sync_dt, t_end=t_end, corr_p=corr_p, corr_m=corr_m, nk_chain=nk_chain,
                   stream=stream, msd=msd)
    return g, o
