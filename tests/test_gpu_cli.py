"""The gpu_DSM command line (CLI/main.cu:20-56 surface) end to end on the GPU:
input.dat in the working directory, tau.dat / G.dat / MSD.dat outputs, -s / -l
conformation files and -distr histograms, named by job_ID like the reference
(common/job_ID.h)."""
import subprocess
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parent.parent
CLI = ROOT / "gpu_dsm_gb300" / "gpu_DSM"


def write_input(d: Path, *, beta=1.0, nk=30, n=256, kappa=(0.0,) * 9, cd=1, pd=0, eq=1, sync=1.0, t_end=100.0):
    lines = [f"\t{beta}", f"\t{nk}", f"\t{n}", "\t" + "\t".join(str(k) for k in kappa), f"\t{cd}", f"\t{pd}",
             f"\t{eq}", f"\t{sync}", f"\t{t_end}", "", "! input file written by the test"]
    (d / "input.dat").write_text("\n".join(lines) + "\n")


def run(d: Path, *args):
    r = subprocess.run([str(CLI), *map(str, args)], cwd=d, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    return r.stdout


def table(p: Path) -> np.ndarray:
    return np.loadtxt(p, ndmin=2)


def test_cli_gt_and_files(dsm_mod, tmp_path):
    write_input(tmp_path, eq=1, t_end=200.0)
    run(tmp_path, 3, "-s", "conf.bin", "-distr")
    g = table(tmp_path / "G_3.dat")
    assert g.shape[1] == 2 and g[0, 0] == 0 and g[0, 1] > 0
    assert (tmp_path / "conf.bin").stat().st_size > 256 * 16
    for name in ("distr_Z.dat", "distr_N.dat", "distr_Q.dat"):  # ensemble.cu:356-484 names
        assert (tmp_path / name).exists(), name
    z = table(tmp_path / "distr_Z.dat")
    assert abs(z[:, 1].sum() - 1.0) < 1e-4


def test_cli_msd(dsm_mod, tmp_path):
    write_input(tmp_path, eq=2, t_end=200.0)
    run(tmp_path, 0)
    m = table(tmp_path / "MSD.dat")
    assert m[0, 1] == 0.0 and np.all(np.diff(m[1:10, 1]) > 0)


def test_cli_flow_and_load(dsm_mod, tmp_path):
    kap = (0.0, 1.0e-3, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0)
    write_input(tmp_path, kappa=kap, eq=0, sync=5.0, t_end=50.0)
    run(tmp_path, 1, "-s", "a.bin")
    tau = table(tmp_path / "tau_1.dat")
    assert tau.shape[0] >= 10 and np.isclose(tau[-1, 0], 50.0)
    # restart from the saved conformations
    run(tmp_path, 2, "-l", "a.bin")
    assert table(tmp_path / "tau_2.dat").shape[0] >= 10


def test_cli_flow_outputs_match_library(dsm_mod, tmp_path):
    """tau.dat of a flow run (100 outputs, so more than one series replay)
    holds the stress of one dsm_advance + dsm_stress per output time, to the
    6 significant digits the driver prints."""
    kap = (0.0, 2.0e-3, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0)
    write_input(tmp_path, nk=30, n=256, kappa=kap, eq=0, sync=0.5, t_end=50.0)
    run(tmp_path, 5)
    tau = table(tmp_path / "tau_5.dat")
    e = dsm_mod.Ensemble(nk=30, n_chains=256, kappa=kap, seed=5, sync_dt=0.5, t_end=50.0)
    e.init_equilibrium()
    times, rows = [], []
    t = 0.0
    while t < 50.0:
        e.advance(t + 0.5)
        times.append(t + 0.5)
        rows.append(e.stress()[0])
        t += 0.5
    assert tau.shape == (100, 9)
    assert np.allclose(tau[:, 0], times, rtol=1e-6, atol=0)
    assert np.allclose(tau[:, 1:], np.array(rows, np.float64), rtol=1e-5, atol=0)


def test_cli_gex_background(dsm_mod, tmp_path):
    """pd_flag = 1 reads polydisp.dat (a b mp Mk) like the reference driver."""
    write_input(tmp_path, pd=1, eq=1, t_end=100.0)
    (tmp_path / "polydisp.dat").write_text("\t1.0\n\t1.0\n\t1000\n\t100\n")
    run(tmp_path, 0)
    assert table(tmp_path / "G.dat")[0, 1] > 0
