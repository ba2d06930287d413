"""End to end through the drop-in's file path, as the reference's drivers run.

A C driver with invert.c's call sequence (tests/drivers/invert_driver.c:
parameter file, ILDG gauge configuration, the twelve columns of an HMC
source file, GCR on Q with iterative refinement, invert.c:170-294) is
compiled against include/qcd.h and linked with the library. It writes each
solution as an ETMC LIME file; the oracle recomputes every solution's FP64
true residual |src - Q sol| / |src| on the CPU. The input files come from the
format models that the host tests pin to the reference's own readers.
"""
import os
import subprocess

import numpy as np
import pytest

import qcd_gb300 as q
from tests import legacy_formats, lime_util
from tests.conftest import EPS_PLAQ_060

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
TH = (np.pi, 0.0, 0.0, 0.0)


def test_invert_driver_end_to_end(gpu, orc, tmp_path):
    L = (8, 4, 4, 6)  # T, X, Y, Z
    kappa, mu, max_res = 0.15, 0.01, 1e-10
    u = orc.gauge_synthetic(L, 21, EPS_PLAQ_060)
    cols = [orc.gaussian_spinor(L, 300 + k) for k in range(12)]
    V = int(np.prod(L))
    cols[4] = np.zeros((V, 4, 3, 2))
    cols[4][5, 1, 1, 0] = 1.0  # one point-source column
    conf, src, sol = tmp_path / "conf.lime", tmp_path / "prop.hmc", tmp_path / "prop.sol"
    conf.write_bytes(lime_util.ildg_file(u, L))
    src.write_bytes(legacy_formats.hmc_file(cols, L, kappa=kappa, mu=mu))
    ini = tmp_path / "invert.ini"
    ini.write_text(f"<processors_txyz>1 1 1 1</processors_txyz>\n<lattice_txyz>{' '.join(map(str, L))}</lattice_txyz>\n"
                   f"<source_type>HMC_PROPAGATOR</source_type>\n<source>{src}</source>\n"
                   f"<solution_type>LIME</solution_type>\n<solution>{sol}</solution>\n<cfg_name>{conf}</cfg_name>\n"
                   f"<N_restart>32</N_restart>\n<kappa>{kappa}</kappa>\n<mu>{mu}</mu>\n<max_res>{max_res}</max_res>\n")
    exe = tmp_path / "invert_driver"
    subprocess.run(["gcc", "-std=gnu99", "-O2", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "drivers", "invert_driver.c"), "-o", str(exe), q.LIB_PATH, "-lm",
                    f"-Wl,-rpath,{os.path.dirname(q.LIB_PATH)}"], check=True)
    out = subprocess.run([str(exe), str(ini)], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stdout + out.stderr
    lines = out.stdout.split("\n")
    plaq = float([x for x in lines if x.startswith("plaquette")][0].split()[1])
    assert abs(plaq - orc.plaquette(u, L)) <= 1e-12
    assert sum(x.startswith("column") for x in lines) == 12
    for c in range(12):
        recs = lime_util.parse((tmp_path / f"prop.sol.{c:02d}").read_bytes())
        assert [r[0] for r in recs] == ["propagator-type", "etmc-propagator-format", "scidac-binary-data"]
        x = lime_util.etmc_array(recs[2][3], L)
        res = orc.true_residual(x, cols[c], u, L, TH, kappa, mu, op="Q")
        assert res <= 1.01 * max_res, (c, res)


def test_invert_driver_reports_a_missing_source(gpu, orc, tmp_path):
    """a source file that cannot be read ends the driver with EXIT_FAILURE, as
    invert.c's exit(EXIT_FAILURE) after qcd_getVector"""
    L = (4, 4, 4, 4)
    conf = tmp_path / "conf.lime"
    conf.write_bytes(lime_util.ildg_file(orc.gauge_synthetic(L, 22, EPS_PLAQ_060), L))
    ini = tmp_path / "invert.ini"
    ini.write_text(f"<lattice_txyz>4 4 4 4</lattice_txyz>\n<source>{tmp_path / 'missing'}</source>\n"
                   f"<solution>{tmp_path / 'sol'}</solution>\n<cfg_name>{conf}</cfg_name>\n"
                   "<N_restart>8</N_restart>\n<kappa>0.12</kappa>\n<mu>0.0</mu>\n")
    exe = tmp_path / "invert_driver"
    subprocess.run(["gcc", "-std=gnu99", "-O2", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "drivers", "invert_driver.c"), "-o", str(exe), q.LIB_PATH, "-lm",
                    f"-Wl,-rpath,{os.path.dirname(q.LIB_PATH)}"], check=True)
    out = subprocess.run([str(exe), str(ini)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 1
    assert "Cannot open" in out.stderr
