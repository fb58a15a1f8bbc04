"""The drop-in boundary seen by compiled callers.

Three programs under tests/abi/ are compiled and linked against libgpudsm.so:
- gui_caller.cpp declares main_cuda itself with C++ linkage, exactly as the
  reference's GUI does (GUI/main.cpp:22, GUI/mainwindow.cpp:47);
- c_caller.c is a C11 caller of the handle API (include/dsm.h);
- ref_api_caller.cpp calls the reference's own entry points and globals
  (include/dsm_reference.h: common/ensemble.h:37-77,
  common/ensemble_call_block.h:55-75) the way common/main_cuda.cu does.
Without a GPU they must compile, link and find every symbol; on the GPU
their results must equal the handle API driven through ctypes bit for bit
(chains, clocks, events), and G(t) / stress to the printed precision."""
import re
import struct
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
ABI = ROOT / "tests" / "abi"
INC = ROOT / "include"
PKG = ROOT / "gpu_dsm_gb300"


def _build(tmp: Path, src: str, lang: str) -> Path:
    exe = tmp / Path(src).stem
    cc = ["gcc", "-std=c11"] if lang == "c" else ["g++", "-std=c++17"]
    cmd = [*cc, "-Wall", "-Werror", "-I", str(INC), str(ABI / src), "-o", str(exe), "-L", str(PKG), "-lgpudsm",
           f"-Wl,-rpath,{PKG}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return exe


@pytest.fixture(scope="module")
def progs(dsm_mod, tmp_path_factory):
    tmp = tmp_path_factory.mktemp("abi")
    return {"gui": _build(tmp, "gui_caller.cpp", "c++"), "c": _build(tmp, "c_caller.c", "c"),
            "ref": _build(tmp, "ref_api_caller.cpp", "c++")}


def test_callers_compile_and_link(progs):
    """C, GUI-style C++ and reference-API C++ callers link against the library."""
    for exe in progs.values():
        assert exe.exists()


def test_reference_symbols_exported(dsm_mod):
    """main_cuda with both linkages and the reference's ensemble.h /
    ensemble_call_block.h functions and globals are in the dynamic symbol table."""
    out = subprocess.run(["nm", "-D", "--defined-only", str(dsm_mod.lib_path())], capture_output=True,
                         text=True).stdout
    syms = {ln.split()[-1] for ln in out.splitlines() if ln.strip()}
    assert "main_cuda" in syms and "_Z9main_cudaPbiPcS0_ibPi" in syms
    demangled = subprocess.run(["c++filt"], input="\n".join(sorted(syms)), capture_output=True, text=True).stdout
    names = {re.sub(r"\(.*", "", s) for s in demangled.splitlines()}
    for f in ("chain_index", "host_chains_init", "gpu_init", "get_chains_from_device", "save_to_file",
              "save_Z_distribution_to_file", "save_N_distribution_to_file", "save_Q_distribution_to_file",
              "load_from_file", "gpu_time_step", "gpu_Gt_PCS", "gpu_clean", "calc_stress", "init_call_block",
              "time_step_call_block", "EQ_time_step_call_block", "get_chain_to_device_call_block",
              "get_chain_from_device_call_block", "calc_stress_call_block", "free_block", "activate_block",
              "deactivate_block", "main_cuda", "N_cha", "NK", "z_max", "Be", "CD_flag", "PD_flag", "kxy",
              "universal_time", "chains", "chain_heads", "job_ID", "dbug"):
        assert f in names, f


# ---------------------------------------------------------------- GPU runs
def _read_ref_file(path: Path, cap: int):
    """Reference conformation file (ensemble.cu:342-354): int N, then per chain
    chain_head, Z float4, Z float."""
    b = path.read_bytes()
    n = struct.unpack_from("i", b, 0)[0]
    off = 4
    Z = np.zeros(n, np.int32)
    time = np.zeros(n, np.float32)
    qn = np.zeros((n, cap, 4), np.float32)
    tau = np.zeros((n, cap), np.float32)
    for i in range(n):
        z, t, _, _ = struct.unpack_from("ifff", b, off)
        Z[i], time[i] = z, t
        off += 16
        qn[i, :z] = np.frombuffer(b, np.float32, 4 * z, off).reshape(z, 4)
        off += 16 * z
        tau[i, :z] = np.frombuffer(b, np.float32, z, off)
        off += 4 * z
    assert off == len(b)
    return Z, time, qn, tau


def _same_chains(a, b, what):
    Za, qa, ta = a
    Zb, qb, tb = b
    assert np.array_equal(Za, Zb), what
    idx = np.arange(qa.shape[1])[None, :] < Za[:, None]
    assert np.array_equal(qa[idx].view(np.uint32), qb[idx].view(np.uint32)), what
    tidx = np.arange(qa.shape[1])[None, :] < (Za - 1)[:, None]
    assert np.array_equal(ta[tidx].view(np.uint32), tb[tidx].view(np.uint32)), what


def _stress_lines(out: str) -> dict:
    d = {}
    for ln in out.splitlines():
        f = ln.split()
        if len(f) == 10 and (f[0].startswith("block") or f[0].startswith("out") or f[0] == "ensemble"):
            d[f[0]] = (np.array([float(v) for v in f[1:9]]), int(f[9]))
    return d


@pytest.mark.gpu
def test_c_caller_matches_handle_api(dsm_mod, progs, tmp_path):
    out = tmp_path / "c.bin"
    r = subprocess.run([str(progs["c"]), "25", "256", "4", "150", str(out)], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    e = dsm_mod.Ensemble(nk=25, n_chains=256, seed=4, eq_type=1, sync_dt=1.0, t_end=150.0, corr_p=16, corr_m=2)
    e.init_equilibrium()
    ev = e.advance(150.0)
    heads, qn, tau = e.get_chains()
    b = out.read_bytes()
    assert struct.unpack_from("Q", b, 0)[0] == ev
    off = 8
    h = np.frombuffer(b, dsm_mod.HEAD_DTYPE, 256, off)
    off += 16 * 256
    q = np.frombuffer(b, np.float32, 256 * 25 * 4, off).reshape(256, 25, 4)
    off += 16 * 256 * 25
    t = np.frombuffer(b, np.float32, 256 * 25, off).reshape(256, 25)
    off += 4 * 256 * 25
    L, p = struct.unpack_from("ii", b, off)
    g = np.frombuffer(b, np.float64, L * p, off + 8).reshape(L, p)
    _same_chains((h["Z"], q, t), (heads["Z"], qn, tau), "C caller")
    assert np.array_equal(h["time"].view(np.uint32), heads["time"].view(np.uint32))
    assert np.array_equal(g, e.gt_raw()[0])


@pytest.mark.gpu
def test_gui_declared_main_cuda_matches_cli(dsm_mod, progs, tmp_path):
    """main_cuda reached through the GUI's C++ declaration writes the same
    G_<id>.dat as the gpu_DSM command line (extern "C" main_cuda)."""
    from test_gpu_cli import write_input
    a, b = tmp_path / "gui", tmp_path / "cli"
    for d in (a, b):
        d.mkdir()
        write_input(d, eq=1, nk=25, n=256, t_end=150.0)
    r = subprocess.run([str(progs["gui"]), "6"], cwd=a, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and "main_cuda=0" in r.stdout, r.stdout + r.stderr
    r = subprocess.run([str(PKG / "gpu_DSM"), "6"], cwd=b, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert (a / "G_6.dat").read_text() == (b / "G_6.dat").read_text()
    assert len((a / "G_6.dat").read_text().splitlines()) > 20


@pytest.mark.gpu
def test_reference_api_gt_and_call_blocks(dsm_mod, progs, tmp_path):
    """host_chains_init -> gpu_init -> gpu_Gt_PCS -> save_to_file / calc_stress,
    then init_call_block -> EQ_time_step_call_block -> calc_stress_call_block
    on two blocks, against the handle API."""
    nk, n, seed, t_end, s = 25, 256, 5, 150.0, 5
    r = subprocess.run([str(progs["ref"]), "gt", str(nk), str(n), str(seed), str(t_end), str(s), "0"],
                       cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    st = _stress_lines(r.stdout)
    # the whole ensemble through gpu_Gt_PCS equals dsm_advance on a handle
    e = dsm_mod.Ensemble(nk=nk, n_chains=n, seed=seed, eq_type=1, sync_dt=1.0, t_end=t_end, corr_levels=s)
    e.init_equilibrium()
    e.advance(t_end)
    heads, qn, tau = e.get_chains()
    Z, time, q, t = _read_ref_file(tmp_path / "ens.bin", nk)
    _same_chains((Z, q, t), (heads["Z"], qn, tau), "gpu_Gt_PCS")
    assert np.array_equal(time.view(np.uint32), heads["time"].view(np.uint32))
    tg, G = e.gt()
    gf = np.loadtxt(tmp_path / f"G_{seed}.dat", ndmin=2)
    assert gf.shape[0] == len(G)
    assert np.array_equal(gf[:, 0], tg) and np.allclose(gf[:, 1], G, rtol=1e-5, atol=0)
    sp, cnt = e.stress()
    assert cnt == n and np.allclose(st["ensemble"][0], sp, rtol=1e-6, atol=1e-7)
    # the call blocks equal handles loaded with the same host state at global chain offsets
    Zi, timei, qi, ti = _read_ref_file(tmp_path / "blocks_in.bin", nk)
    Zb, timeb, qb, tb = _read_ref_file(tmp_path / "blocks.bin", nk)
    half = n // 2
    for k, (lo, hi) in enumerate(((0, half), (half, n))):
        h = np.zeros(hi - lo, dsm_mod.HEAD_DTYPE)
        h["Z"], h["time"] = Zi[lo:hi], timei[lo:hi]
        x = dsm_mod.Ensemble(nk=nk, n_chains=hi - lo, seed=seed, eq_type=1, sync_dt=1.0, t_end=t_end + 100.0,
                             corr_levels=s, chain_offset=lo)
        x.set_chains(h, qi[lo:hi], ti[lo:hi])
        x.advance(t_end + 100.0)
        hx, qx, tx = x.get_chains()
        _same_chains((Zb[lo:hi], qb[lo:hi], tb[lo:hi]), (hx["Z"], qx, tx), f"call block {k}")
        sx, cx = x.stress()
        assert st[f"block{k}"][1] == cx and np.allclose(st[f"block{k}"][0], sx, rtol=1e-6, atol=1e-7)


@pytest.mark.gpu
def test_reference_api_flow(dsm_mod, progs, tmp_path):
    """gpu_time_step + calc_stress at every output (the reference's flow loop,
    main_cuda.cu:122-140) against dsm_advance + dsm_stress."""
    nk, n, seed, kxy, dt, nout = 50, 256, 8, 2.0e-3, 10.0, 5
    r = subprocess.run([str(progs["ref"]), "flow", str(nk), str(n), str(seed), str(kxy), str(dt), str(nout)],
                       cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    st = _stress_lines(r.stdout)
    e = dsm_mod.Ensemble(nk=nk, n_chains=n, seed=seed, kappa=(0.0, kxy, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0))
    e.init_equilibrium()
    for k in range(1, nout + 1):
        e.advance(k * dt)
        sp, cnt = e.stress()
        assert st[f"out{k}"][1] == cnt and np.allclose(st[f"out{k}"][0], sp, rtol=1e-6, atol=1e-7), k
    heads, qn, tau = e.get_chains()
    Z, _, q, t = _read_ref_file(tmp_path / "ens.bin", nk)
    _same_chains((Z, q, t), (heads["Z"], qn, tau), "gpu_time_step")
