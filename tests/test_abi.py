"""The C-ABI library builds, loads without a GPU and exports every entry point
declared in include/dsm.h; GPU calls fail with a status code (no CPU fallback)."""
import ctypes
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def declared_functions():
    src = (ROOT / "include" / "dsm.h").read_text()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"^\s*(?:int|void|const char\*)\s+\**(\w+)\s*\(", src, flags=re.M)
    return sorted(set(names))


def test_header_declares_api():
    names = declared_functions()
    for must in ("dsm_create", "dsm_advance", "dsm_gt", "dsm_stress", "main_cuda", "dsm_set_chains"):
        assert must in names


def test_library_exports_all_symbols(dsm_mod):
    lib = ctypes.CDLL(str(dsm_mod.lib_path()))
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_no_cpu_fallback_without_gpu(dsm_mod):
    import torch

    if torch.cuda.is_available():
        pytest.skip("GPU present")
    with pytest.raises(dsm_mod.DSMError) as e:
        dsm_mod.Ensemble(nk=25, n_chains=8)
    assert e.value.code == -2


def test_invalid_arguments(dsm_mod):
    with pytest.raises(dsm_mod.DSMError) as e:
        dsm_mod.Ensemble(nk=0, n_chains=8)
    assert e.value.code == -3
    with pytest.raises(dsm_mod.DSMError) as e:
        dsm_mod.Ensemble(nk=25, n_chains=8, z_max=5000)
    assert e.value.code == -3


def test_cli_built(dsm_mod):
    assert (ROOT / "gpu_dsm_gb300" / "gpu_DSM").exists()


def test_pcd_export_matches_reference(dsm_mod):
    """dsm_pcd (host code, no GPU) reproduces the reference's compiled p_cd fits."""
    import json

    d = json.loads((ROOT / "tests" / "golden" / "pcd_reference.json").read_text())
    for r in d["rows"]:
        ours = dsm_mod.pcd(r["beta"], r["nk"])
        for k in ("alpha", "tau_0", "tau_max", "tau_d", "g", "normdt"):
            assert ours[k] == pytest.approx(r[k], rel=1e-5, abs=1e-12), (r["beta"], r["nk"], k)
    with pytest.raises(dsm_mod.DSMError):
        dsm_mod.pcd(0.0, 10)


def test_gex_tables_match_reference(dsm_mod):
    """GEX background tables (host code, no GPU) against the reference's own
    make_gamma_table (gamma.cpp:174-263, compiled): same sizes and steps, the
    M/mp table to 1e-5, the CD-weighted one to 1e-3 (p_cd in double here)."""
    import ctypes as C
    import json

    import numpy as np

    L = dsm_mod.load_library()
    L.dsm_gex_table.argtypes = [C.c_float] * 4 + [C.c_double] + [C.c_void_p] * 5
    d = json.loads((ROOT / "tests" / "golden" / "gex_reference.json").read_text())
    assert len(d["rows"]) >= 3
    for r in d["rows"]:
        cap = 200000
        m, md = np.zeros(cap, np.float32), np.zeros(cap, np.float32)
        n, nd = np.array([cap], np.int32), np.array([cap], np.int32)
        info = np.zeros(3)
        assert L.dsm_gex_table(r["a"], r["b"], r["mp"], r["mk"], r["beta"], m.ctypes.data, n.ctypes.data,
                               md.ctypes.data, nd.ctypes.data, info.ctypes.data) == 0
        assert n[0] == r["n"] and nd[0] == r["n_d"]
        assert info[0] == pytest.approx(r["step"], rel=1e-6) and info[1] == pytest.approx(r["step_d"], rel=1e-4)
        ev = r["every"]
        ref_m, ours_m = np.array(r["M"]), m[: n[0]][::ev]
        assert np.all(np.abs(ours_m[1:] - ref_m[1:]) <= 1e-5 * ref_m[1:])
        # the reference's last CD-weighted entry can come from uninitialised memory
        ref_md, ours_md = np.array(r["Md"])[:-1], md[: nd[0]][::ev][: len(r["Md"]) - 1]
        assert np.all(np.abs(ours_md[1:] - ref_md[1:]) <= 1e-3 * ref_md[1:])
