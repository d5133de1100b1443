"""netCDF-3 output/restart of the library, checked with scipy's independent
netCDF-3 reader: the reference's vars.nc layout (src/netcdf_io.h:38-277)."""
import numpy as np
import pytest
from scipy.io import netcdf_file


def test_vars_nc_layout_and_values(qgwlib, tmp_path):
    nl, ny2, nx2, D = 3, 9, 17, 2.5e5
    path = str(tmp_path / "vars.nc")
    w = qgwlib.NcWriter(path, nl, ny2, nx2, D)
    rng = np.random.default_rng(0)
    recs = []
    for r in range(3):
        psi = rng.standard_normal((nl, ny2, nx2))
        q = rng.standard_normal((nl, ny2, nx2)) * 1e-7
        w.write(1000.0 * r, psi, q)
        recs.append((psi, q))
    w.close()
    f = netcdf_file(path, "r", mmap=False)
    assert f.dimensions["t"] is None and f.dimensions["level"] == nl
    assert f.dimensions["y"] == ny2 and f.dimensions["x"] == nx2
    assert list(f.variables.keys()) == ["t", "y", "x", "level", "psi", "q"]
    assert f.variables["psi"].dimensions == ("t", "level", "y", "x")
    assert np.allclose(f.variables["t"][:], [0.0, 1000.0, 2000.0])
    assert np.allclose(f.variables["x"][:], np.arange(nx2) * D)
    assert np.allclose(f.variables["level"][:], np.arange(nl))
    for r, (psi, q) in enumerate(recs):
        assert np.array_equal(f.variables["psi"][r], psi.astype(np.float32))
        assert np.array_equal(f.variables["q"][r], q.astype(np.float32))
    f.close()
    # the library's own reader (restart path): record 2 of q
    back = qgwlib.nc_read(path, "q", (nl, ny2, nx2), rec=2)
    assert np.array_equal(back, recs[2][1].astype(np.float32).astype(np.float64))


def test_restart_reader_accepts_scipy_file(qgwlib, tmp_path):
    path = str(tmp_path / "restart.nc")
    f = netcdf_file(path, "w")
    f.createDimension("t", None)
    f.createDimension("level", 2)
    f.createDimension("y", 5)
    f.createDimension("x", 6)
    v = f.createVariable("q", "f", ("t", "level", "y", "x"))
    tp = f.createVariable("topo", "d", ("t", "y", "x"))
    data = np.arange(60, dtype=np.float32).reshape(1, 2, 5, 6)
    v[:] = data
    tp[:] = np.ones((1, 5, 6)) * 3.5
    f.close()
    q = qgwlib.nc_read(path, "q", (2, 5, 6))
    assert np.array_equal(q, data[0].astype(np.float64))
    assert np.all(qgwlib.nc_read(path, "topo", (5, 6)) == 3.5)
    with pytest.raises(qgwlib.QgwError):
        qgwlib.nc_read(path, "missing", (5, 6))
