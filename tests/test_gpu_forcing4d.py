"""4-D forcing on the GPU (dt_forc_period != 0, src/forcing.h:226-288):
records of q_forcing_3d interpolated linearly in time, added to every layer
as q_forc * dt after the AB3 update (src/timestep.h:152-163).  The
reference's own golden runs (it reads input_vars.nc itself through the
oracle's netCDF reader) are covered by
test_gpu_parity.test_fp64_matches_reference_golden (forcing4d_* cases);
here larger grids against the C port, the compensated path, ensembles, the
refusals and the drop-in driver reading input_vars.nc."""
import os
import subprocess

import numpy as np
import pytest
from scipy.io import netcdf_file

from qgw_gb300 import configs as C
from qgw_gb300.params import write_params
from test_gpu_parity import TOL32C, TOL64, gpu_run, records_layout, rel

pytestmark = pytest.mark.gpu


def forced(p, nrec=4, dt_forc=3600.0, seed=5):
    p = dict(p, dt_forc=dt_forc, dt_forc_period=nrec * dt_forc)
    nl, nyp2, nxp2 = C.halo_shape(p)
    ibc = 1 if p.get("bc_fac", 0.0) == -1 else 0
    rng = np.random.Generator(np.random.PCG64(seed))
    frec = rng.normal(0.0, 1e-11, size=(nrec, nl, nyp2 - 2 * ibc, nxp2 - 2 * ibc)).astype(np.float32)
    return p, frec


@pytest.mark.parametrize("bc,nx", [(0.0, 128), (-1.0, 128), (0.0, 96)])
def test_forcing4d_fp64_vs_port(qgwlib, oracle_mod, bc, nx):
    p, frec = forced(dict(C.cfg2(nx, 5), bc_fac=bc))
    q0 = C.noise_ic(p, 41)
    o = oracle_mod.run_port(p, q0, 50, dt_fixed=600.0, forcing_records=frec)
    psi, q, _ = gpu_run(qgwlib, p, q0, 50, 600.0, frec=frec)
    assert rel(q, o["q"]) <= TOL64, rel(q, o["q"])
    assert rel(psi, o["psi"]) <= TOL64, rel(psi, o["psi"])


def test_forcing4d_fp32c_vs_fp64(qgwlib):
    p, frec = forced(C.cfg2(256, 10))
    q0 = C.noise_ic(p, 42)
    psi64, q64, _ = gpu_run(qgwlib, p, q0, 100, 600.0, precision=0, frec=frec)
    psi32, q32, _ = gpu_run(qgwlib, p, q0, 100, 600.0, precision=1, frec=frec)
    assert rel(q32, q64) <= TOL32C, rel(q32, q64)
    assert rel(psi32, psi64) <= TOL32C, rel(psi32, psi64)


def test_forcing4d_ensemble_alone_equals_mix(qgwlib):
    (p1, f1), (p2, f2) = forced(C.cfg1(64), seed=1), forced(C.cfg2(32, 5), nrec=2, seed=2)
    ens = qgwlib.Ensemble([p1, p2], 1)
    for i, (p, f) in enumerate(((p1, f1), (p2, f2))):
        ens.set_forcing_records(i, records_layout(p, f))
        ens.set_q(i, C.noise_ic(p, 60 + i))
        ens.fix_dt(i, p["dt"])
    ens.step(9)
    for i, (p, f) in enumerate(((p1, f1), (p2, f2))):
        psi, q = ens.get(i)
        psi_a, q_a, _ = gpu_run(qgwlib, p, C.noise_ic(p, 60 + i), 9, p["dt"], precision=1, frec=f)
        assert np.array_equal(q, q_a) and np.array_equal(psi, psi_a), i
    ens.close()


def test_forcing4d_refusals(qgwlib):
    with pytest.raises(qgwlib.QgwError) as e:  # dt_forc_period not a multiple of dt_forc
        qgwlib.Run(dict(C.cfg1(64), dt_forc=3600.0, dt_forc_period=5000.0))
    assert e.value.status == -1
    p, _ = forced(C.cfg1(64))
    r = qgwlib.Run(p)
    r.set_q(C.noise_ic(p, 1))
    with pytest.raises(qgwlib.QgwError) as e:  # records not set
        r.step(1)
    assert e.value.status == -8
    r.close()


def test_driver_reads_input_vars(qgwlib, oracle_mod, tmp_path):
    """The drop-in executable reads the records from input_vars.nc like the
    reference (read_nc of q_forcing_3d), periodic basin (interior files)."""
    from qgw_gb300 import build
    # outputs at the top of the driver loop (src/qg.c:181-199): t = 0 and
    # t = 12 steps, then one more step to tend
    p, frec = forced(dict(C.cfg1(64), bc_fac=-1.0, tend=1200.0 * 13, dt_out=1200.0 * 12))
    q0 = np.zeros(C.halo_shape(p))
    f = netcdf_file(str(tmp_path / "input_vars.nc"), "w")
    f.createDimension("time", None)
    f.createDimension("level", frec.shape[1])
    f.createDimension("y", frec.shape[2])
    f.createDimension("x", frec.shape[3])
    v = f.createVariable("q_forcing_3d", "f", ("time", "level", "y", "x"))
    v[:] = frec
    f.close()
    write_params(str(tmp_path / "params.in"), p)
    r = subprocess.run([build.DRIVER], capture_output=True, text=True, cwd=tmp_path, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    nc = netcdf_file(str(tmp_path / "outdir_0001" / "vars.nc"), "r", mmap=False)
    q_last = nc.variables["q"][-1].astype(np.float64)
    t = nc.variables["t"][:].copy()
    nc.close()
    assert np.allclose(t, [0.0, 1200.0 * 12])
    assert q_last.shape == frec.shape[1:]  # periodic files hold the interior
    o = oracle_mod.run_port(p, q0, 12, dt_fixed=1200.0, forcing_records=frec)
    qo = o["q"][:, 1:-1, 1:-1]
    assert np.abs(q_last - qo).max() <= 1e-6 * np.abs(qo).max()
