"""The qg executable on GB300 (qgw_gb300/driver/qg_gpu.cpp): the reference's
driver loop with params.in, outdir_NNNN/, restart.nc and vars.nc."""
import os
import subprocess

import numpy as np
import pytest
from scipy.io import netcdf_file

from qgw_gb300 import configs as C
from qgw_gb300.params import write_params


def test_driver_binary_links(qgwlib):
    from qgw_gb300 import build
    assert os.path.exists(build.DRIVER)


def test_missing_params_file(qgwlib, tmp_path):
    from qgw_gb300 import build
    r = subprocess.run([build.DRIVER, str(tmp_path / "nope.in")], capture_output=True, text=True, cwd=tmp_path)
    assert "not found" in r.stdout and r.returncode != 0


@pytest.mark.gpu
def test_driver_run_matches_oracle(qgwlib, oracle_mod, tmp_path):
    from qgw_gb300 import build
    p = dict(C.cfg1(64), tend=12000.0 * 3, dt_out=12000.0)
    q0 = C.noise_ic(p, 77)
    # restart.nc carrying the initial q (the reference's restart path)
    f = netcdf_file(str(tmp_path / "restart.nc"), "w")
    f.createDimension("t", None)
    f.createDimension("level", 3)
    f.createDimension("y", 65)
    f.createDimension("x", 65)
    v = f.createVariable("q", "f", ("t", "level", "y", "x"))
    v[:] = q0[None].astype(np.float32)
    f.close()
    write_params(str(tmp_path / "params.in"), p)
    r = subprocess.run([build.DRIVER], capture_output=True, text=True, cwd=tmp_path, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    out = tmp_path / "outdir_0001"
    assert (out / "params.in").exists()
    nc = netcdf_file(str(out / "vars.nc"), "r", mmap=False)
    t = nc.variables["t"][:].copy()
    q_last = nc.variables["q"][-1].astype(np.float64)
    psi_last = nc.variables["psi"][-1].astype(np.float64)
    nc.close()
    assert np.allclose(t, [0.0, 12000.0, 24000.0])
    # the oracle from the same float32 restart, 20 steps of 1200 s
    q0f = q0.astype(np.float32).astype(np.float64)
    o = oracle_mod.run_port(p, q0f, 20, dt_fixed=1200.0)
    assert np.abs(q_last - o["q"]).max() <= 1e-6 * np.abs(o["q"]).max()
    assert np.abs(psi_last - o["psi"]).max() <= 1e-6 * np.abs(o["psi"]).max()
