"""GUI-equivalent parameter mapping (GUI/mainwindow.cpp:556-640, 823-839):
CFSM/FSM strand counts, tau_d-based run lengths, flow patterns of
GUI/flow.txt, Wi, and the input.dat / polydisp.dat files it writes."""
import math

import numpy as np
import pytest

from gpu_dsm_gb300 import setup_run as sr


def test_cfsm_equilibrium(tmp_path):
    p = sr.map_parameters(mw_kg_mol=100.0, mk_g_mol=100.0, model="CFSM", beta=1.0, n_chains=512)
    assert p["nk"] == math.ceil(1000 / 0.56) and p["beta"] == 1.0
    assert p["eq_type"] == 1 and p["sync_dt"] == 1.0
    assert p["t_end"] == pytest.approx(0.0740131 * p["nk"] ** 3.18363)
    path = sr.write_input(tmp_path, p)
    vals = path.read_text().split()
    assert float(vals[0]) == 1.0 and int(vals[1]) == p["nk"] and int(vals[2]) == 512
    assert [float(v) for v in vals[3:12]] == [0.0] * 9 and vals[12:15] == ["1", "0", "1"]


def test_fsm_tau_d_matches_pcd_fit(dsm_mod):
    p = sr.map_parameters(mw_kg_mol=20.0, mk_g_mol=200.0, model="FSM", beta=2.0)
    assert p["nk"] == 100 and p["beta"] == 2.0
    assert p["tau_d"] == pytest.approx(dsm_mod.pcd(2.0, 100)["tau_d"], rel=1e-6)


@pytest.mark.parametrize("flow,row", [("inception", (0, 1, 0, 0, 0, 0, 0, 0, 0)),
                                      ("uniaxial", (-0.5, 0, 0, 0, -0.5, 0, 0, 0, 1))])
def test_flow_mapping(tmp_path, flow, row):
    p = sr.map_parameters(mw_kg_mol=10.0, mk_g_mol=100.0, model="CFSM", flow=flow, rate=1e-3, strain=30.0,
                          polydisp=(1.0, 1.0, 1000.0, 100.0))
    assert np.allclose(p["kappa"], np.array(row) * 1e-3)
    assert p["t_end"] == 30000.0 and p["sync_dt"] == 30.0 and p["eq_type"] == 0
    assert p["Wi"] == pytest.approx(1e-3 * p["tau_d"])
    sr.write_input(tmp_path, p)
    assert [float(v) for v in (tmp_path / "polydisp.dat").read_text().split()] == [1.0, 1.0, 1000.0, 100.0]
    assert (tmp_path / "input.dat").read_text().split()[13] == "1"  # pd_flag


def test_short_flow_sync_floor():
    p = sr.map_parameters(mw_kg_mol=10.0, mk_g_mol=100.0, flow="planar", rate=0.1, strain=5.0)
    assert p["t_end"] == 50.0 and p["sync_dt"] == 1.0
