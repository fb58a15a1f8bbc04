"""dsm_advance_noalloc: the allocation-free time step for callers that cannot
call cudaMalloc/cudaFree around a step (a serving loop or host framework that
owns every byte of device memory through its own allocator or budget, or a
loop that cannot take the device-wide synchronisation those calls imply).

The test owns the device buffers (allocated here with torch); the entry point
only uses them and its static scratch array.  Its results must equal those of
the allocating entry point dsm_advance on the same inputs, bit for bit, on two
calls in a row.  This file is collected last on purpose."""
import ctypes as C

import numpy as np
import pytest

STATE_DTYPE = np.dtype([("Z", np.int32), ("stall_flag", np.int32), ("scale", np.int32), ("dt_prev", np.float32),
                        ("time_ticks", np.int64), ("steps", np.uint64), ("hash", np.uint64),
                        ("next_sample", np.int64), ("nk", np.int32), ("pad", np.int32, 3)])
assert STATE_DTYPE.itemsize == 64


def _bind(dsm_mod):
    lib = dsm_mod.load_library()
    lib.dsm_advance_noalloc.argtypes = [C.POINTER(dsm_mod.api.DsmParams), C.c_void_p, C.c_void_p, C.c_void_p,
                                        C.c_void_p, C.c_double, C.c_int64, C.c_void_p, C.POINTER(C.c_uint64)]
    lib.dsm_advance_noalloc.restype = C.c_int
    lib.dsm_noalloc_last_error.argtypes = []
    lib.dsm_noalloc_last_error.restype = C.c_char_p
    return lib


def test_noalloc_rejects_oversize(dsm_mod):
    """nk beyond DSM_NOALLOC_MAX_NK is refused before any device work."""
    lib = _bind(dsm_mod)
    p = dsm_mod.api.DsmParams()
    p.beta, p.nk, p.n_chains, p.cd_flag = 1.0, 4096, 8, 1
    buf = C.c_void_p(1)  # never dereferenced: the size check comes first
    rc = lib.dsm_advance_noalloc(C.byref(p), buf, buf, buf, None, 10.0, -1, None, None)
    assert rc == -3
    assert b"exceeds the no-allocation limit" in lib.dsm_noalloc_last_error()


@pytest.mark.parametrize("eq_type", [1, 2])
def test_noalloc_rejects_correlator(dsm_mod, eq_type):
    """Parameters for which dsm_create would run a G(t) (eq_type 1) or MSD
    (eq_type 2) correlator are refused before any device work."""
    lib = _bind(dsm_mod)
    p = dsm_mod.api.DsmParams()
    p.beta, p.nk, p.n_chains, p.cd_flag = 1.0, 25, 8, 1
    p.eq_type, p.sync_dt, p.t_end = eq_type, 1.0, 10.0
    buf = C.c_void_p(1)  # never dereferenced: the correlator check comes first
    rc = lib.dsm_advance_noalloc(C.byref(p), buf, buf, buf, None, 10.0, -1, None, None)
    assert rc == -3
    assert b"correlator" in lib.dsm_noalloc_last_error()


@pytest.mark.gpu
@pytest.mark.parametrize("kappa,nk,n", [((0.0,) * 9, 50, 512), ((0.0, 2.0e-3, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0), 50, 512),
                                        ((0.0,) * 9, 2000, 64)])
def test_noalloc_matches_dsm_advance(dsm_mod, kappa, nk, n):
    import torch

    lib = _bind(dsm_mod)
    ens = dsm_mod.Ensemble(nk=nk, n_chains=n, seed=3, kappa=kappa)
    ens.init_equilibrium()
    heads, qn, tau = ens.get_chains()
    ext = ens.get_ext()
    st = np.zeros(n, STATE_DTYPE)
    st["Z"], st["stall_flag"], st["scale"], st["dt_prev"] = heads["Z"], ext["stall"], ext["S"], ext["dt_prev"]
    st["time_ticks"], st["steps"], st["hash"], st["nk"] = ext["T"], ext["step"], ext["hash"], nk
    d_qn = torch.from_numpy(qn.copy()).cuda()
    d_tau = torch.from_numpy(tau.copy()).cuda()
    d_st = torch.from_numpy(st.view(np.uint8).copy()).cuda()
    d_stress = torch.zeros(n * 8, dtype=torch.float32, device="cuda")
    flow = any(k != 0 for k in kappa)
    idx = np.arange(nk)[None, :]
    for t_end in (30.0, 75.0):  # two calls in a row, the second continues the first
        ev_ref = ens.advance(t_end)
        torch.cuda.synchronize()
        ev = C.c_uint64(0)
        rc = lib.dsm_advance_noalloc(C.byref(ens.params), C.c_void_p(d_qn.data_ptr()), C.c_void_p(d_tau.data_ptr()),
                                     C.c_void_p(d_st.data_ptr()), C.c_void_p(d_stress.data_ptr()) if flow else None,
                                     t_end, -1, None, C.byref(ev))
        assert rc == 0, lib.dsm_noalloc_last_error()
        torch.cuda.synchronize()
        assert ev.value == ev_ref
        h_ref, q_ref, t_ref = ens.get_chains()
        x_ref = ens.get_ext()
        got = d_st.cpu().numpy().view(STATE_DTYPE)
        Z = got["Z"]
        assert np.array_equal(Z, h_ref["Z"])
        for k_got, k_ref in (("stall_flag", "stall"), ("scale", "S"), ("time_ticks", "T"), ("steps", "step"),
                             ("hash", "hash")):
            assert np.array_equal(got[k_got], x_ref[k_ref]), k_got
        assert np.array_equal(got["dt_prev"].view(np.uint32), x_ref["dt_prev"].view(np.uint32))
        mq = idx < Z[:, None]
        mt = idx < (Z[:, None] - 1)
        q_got = d_qn.cpu().numpy()
        t_got = d_tau.cpu().numpy()
        assert np.array_equal(q_got[mq].view(np.uint32), q_ref[mq].view(np.uint32))
        assert np.array_equal(t_got[mt].view(np.uint32), t_ref[mt].view(np.uint32))
        if flow:
            s_ref, cnt = ens.stress()
            s = d_stress.cpu().numpy().reshape(n, 8).astype(np.float64)
            ok = (got["stall_flag"] == 0) & ~np.isnan(s[:, 0])
            assert ok.sum() == cnt
            mean = s[ok].mean(axis=0)
            assert np.allclose(mean, s_ref, rtol=1e-6, atol=1e-7), (mean, s_ref)
    ens.close()
