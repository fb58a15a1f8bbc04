"""The phase-clock debug build stays out of the product library.

gpu_dsm_gb300/phases.py builds libgpudsm_phases.so (-DDSM_PHASE_CLOCKS) to
attribute the step kernel's cycles to the phases of its event loop; the
library the package loads must not carry those clock reads."""
import ctypes as C

import pytest


def test_product_library_has_no_phase_clocks(dsm_mod):
    lib = C.CDLL(str(dsm_mod.lib_path()))
    for sym in ("dsm_phase_read", "dsm_phase_clear"):
        with pytest.raises(AttributeError):
            getattr(lib, sym)


def test_phase_tool_parses_without_cases():
    from gpu_dsm_gb300 import phases

    assert phases.main(["--cases", ""]) == 0
    assert len(phases.NAMES) == 12
