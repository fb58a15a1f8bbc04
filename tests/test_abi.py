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
