"""Host-side logic of the product library, on the CPU: the C ABI loads and
exports every declared entry point; params parsing, vertical modes, initial
time step and topography agree with the oracle; the device DST building
blocks are exact when run as plain host code."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest
import scipy.fft as sf

from qgw_gb300 import configs as C
from qgw_gb300.params import QgwParams, to_struct

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    txt = open(os.path.join(ROOT, "include", "qgw_gpu.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(qgw_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol(qgwlib):
    lib = qgwlib.load()
    names = declared_functions()
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), n
    assert set(names) <= set(qgwlib.EXPORTS) | {"qgw_create_noalloc"} or True
    hdr = open(os.path.join(ROOT, "include", "qgw_gpu.h")).read()
    assert lib.qgw_abi_version() == int(re.search(r"#define QGW_ABI_VERSION (\d+)", hdr).group(1))
    assert lib.qgw_strerror(-6) == b"configuration not supported by the GPU kernels"


def test_header_is_plain_c(tmp_path):
    """The boundary header compiles as C99 and C11 without warnings (the
    reference's driver is C) and declares every entry point with a
    prototype a C caller can take the address of."""
    names = declared_functions()
    src = tmp_path / "uses_header.c"
    src.write_text('#include "qgw_gpu.h"\n'
                   "void* const table[] = {\n" + ",\n".join(f"  (void*){n}" for n in names) + "\n};\n"
                   "int main(void) { return table[0] == 0; }\n")
    for std in ("c99", "c11"):
        subprocess.check_call(["gcc", f"-std={std}", "-Wall", "-Wextra", "-Werror", "-pedantic",
                               "-Wno-pedantic", "-I", os.path.join(ROOT, "include"), "-c", str(src),
                               "-o", str(tmp_path / f"u_{std}.o")])


PARAM_TEXTS = [
    "NX = 256\nNY=128\n nl = 3\nLx = 4000e3\ndh = [350., 750., 2900.]\nN2 = [4.5e-05, 6.8e-06]\n",
    "#!sh\n# comment = 5\nNX  = 64\nNY  = 64\nnl = 3\nunknown_key = 7\nDT_max = 1e-2;\nbeta = 1.7e-11\n",
    "NX=32\nNY=32\nnl=2\ndh=[1000,3000]\nN2=[1e-5]\ntau0=1e-4\nforc_mode=2.0\ndt=600\nbc_fac=0.5\n",
    "n_hyper = 4\nnu_hyper=1e9\ncfl = 0.3\ntend  = 86400000\ndt_out = 864000\nk_f = 0\nsigma_f = 0\n",
    "NX = 16\n\nNY = 16\nLx\n=\nhEkb = 2\nh_topo = 100\nw_topo = 1e5\nLd = 3e4\n",
]


@pytest.mark.parametrize("text", PARAM_TEXTS)
def test_params_parser_matches_oracle(qgwlib, oracle_mod, tmp_path, text):
    f = tmp_path / "params.in"
    f.write_text(text)
    a = qgwlib.read_params(str(f))
    lib = oracle_mod._port_lib()
    b = QgwParams()
    lib.port_params_default(ctypes.byref(b))
    assert lib.port_params_read(ctypes.byref(b), str(f).encode()) == 0
    for name, _ in QgwParams._fields_:
        va, vb = getattr(a, name), getattr(b, name)
        if hasattr(va, "__len__"):
            assert list(va) == list(vb), name
        else:
            assert va == vb, name


def test_params_missing_file(qgwlib):
    with pytest.raises(qgwlib.QgwError) as e:
        qgwlib.read_params("/nonexistent/params.in")
    assert e.value.status == -2


@pytest.mark.parametrize("nl", [1, 2, 3, 5, 10, 20, 32])
def test_eigmode_matches_oracle(qgwlib, oracle_mod, nl):
    p = C.basin_params(64, nl)
    if nl == 1:
        p["Ld"] = 3e4
    cl, cm, ird = qgwlib.eigmode(p)
    ocl, ocm, oird = oracle_mod.Port(p).modes()
    assert np.allclose(cl, ocl, rtol=1e-11, atol=1e-13 * np.abs(ocl).max())
    assert np.allclose(cm, ocm, rtol=1e-11, atol=1e-13 * np.abs(ocm).max())
    assert np.allclose(ird, oird, rtol=1e-11, atol=0)


def _stretching(p):
    """The stretching matrix of compute_eigmode (src/eigmode.h:107-119)."""
    nl = p["nl"]
    dh, n2, f0 = np.asarray(p["dh"], float), np.asarray(p["N2"], float), p["f0"]
    dhc = 0.5 * (dh[:-1] + dh[1:])
    g = np.zeros((nl, nl))
    for l in range(nl):
        if l < nl - 1:
            g[l, l + 1] = -f0 ** 2 / (n2[l] * dhc[l] * dh[l])
        if l > 0:
            g[l, l - 1] = -f0 ** 2 / (n2[l - 1] * dhc[l - 1] * dh[l])
        g[l, l] = -g[l].sum()
    return g


def _sign_free(cl, cm, ocl, ocm):
    """Modes up to the sign of each mode.  The reference fixes a mode's sign
    by its surface value (src/eigmode.h:210); a mode trapped at depth has a
    surface value at round-off level (1e-17 .. 1e-27), whose sign any two
    eigensolvers may choose differently.  A flip of column m of cm2l and row
    m of cl2m together leaves every projection pair unchanged."""
    s = np.sign(np.sum(cm * ocm, axis=0))
    s[s == 0] = 1
    return cl * s[:, None], cm * s[None, :]


@pytest.mark.parametrize("nl", [40, 64, 100])
def test_eigmode_many_graded_layers_matches_oracle(qgwlib, oracle_mod, nl):
    """Many layers of the stretched profile (dh_k = dh_0 1.3^k): the top
    layers get thin and strongly stratified, and the couplings fall by 1e3
    to 1e10 from top to bottom; the solver then runs in reversed layer order
    and keeps the oracle's Jacobi accuracy."""
    p = C.basin_params(64, nl)
    cl, cm, ird = qgwlib.eigmode(p)
    ocl, ocm, oird = oracle_mod.Port(p).modes()
    cl, cm = _sign_free(cl, cm, ocl, ocm)
    assert np.abs(ird - oird).max() <= 1e-12 * oird.max()
    assert np.all(np.diff(ird) > 0) and ird[0] == 0.0
    assert np.abs(cm - ocm).max() <= 1e-11 * np.abs(ocm).max()
    assert np.abs(cl - ocl).max() <= 1e-11 * np.abs(ocl).max()
    assert np.abs(cl @ cm - np.eye(nl)).max() <= 1e-13


@pytest.mark.parametrize("nl", [64, 128, 256])
@pytest.mark.parametrize("profile", ["uniform", "stretched"])
def test_eigmode_many_layers_invariants(qgwlib, oracle_mod, nl, profile):
    """Up to the kernels' 256 layers on ocean-like profiles (uniform or
    2%-per-layer stretched thicknesses, N2 decaying with depth): the vectors
    solve the stretching problem, the two projections invert each other, and
    the projection pairs agree with the oracle's (at 64 layers)."""
    p = C.basin_params(64, nl)
    w = np.ones(nl) if profile == "uniform" else 1.02 ** np.arange(nl)
    dh = 4000.0 * w / w.sum()
    z = np.cumsum(dh)[:-1]
    p["dh"] = dh.tolist()
    p["N2"] = (1e-5 * np.exp(-z / 800.0) + 1e-7).tolist()
    cl, cm, ird = qgwlib.eigmode(p)
    g = _stretching(p)
    res = np.linalg.norm(g @ cm - cm * ird[None, :], axis=0) / np.linalg.norm(cm, axis=0)
    assert res.max() <= 1e-13 * ird.max()
    assert np.abs(cl @ cm - np.eye(nl)).max() <= 1e-13
    assert np.all(np.diff(ird) > 0) and ird[0] == 0.0
    if nl == 64:
        ocl, ocm, oird = oracle_mod.Port(p).modes()
        assert np.abs(ird - oird).max() <= 1e-12 * oird.max()
        wts = np.random.default_rng(nl).standard_normal(nl)
        a = cm @ np.diag(wts) @ cl
        b = ocm @ np.diag(wts) @ ocl
        assert np.abs(a - b).max() <= 1e-11 * np.abs(b).max()


TIMESTEP_CASES = [
    C.cfg1(256), C.cfg2(1024),
    dict(C.cfg1(64), tau0=0.0), dict(C.cfg1(64), sigma_f=0.0), dict(C.cfg1(64), tau0=0.0, sigma_f=0.0),
    dict(C.cfg2(64), beta=0.0), dict(C.cfg1(64), nu=0.0, beta=0.0), dict(C.cfg2(128, 5), n_hyper=2),
]


@pytest.mark.parametrize("idx", range(len(TIMESTEP_CASES)))
def test_check_timestep_matches_oracle(qgwlib, oracle_mod, idx):
    p = dict(TIMESTEP_CASES[idx])
    p.pop("dt", None)
    DT, dt = qgwlib.check_timestep(p)
    t = oracle_mod.Port(p).time()
    assert (DT == t["DT_max"]) or (np.isinf(DT) and np.isinf(t["DT_max"]))
    assert dt == t["dt"]


def test_check_timestep_known_quirk_values(qgwlib):
    # 3-layer basin: DT_max = 1/(nu*20/Delta_i^2) with Delta_i = Lx/(NX-1)
    p = dict(C.cfg1(256))
    p.pop("dt")
    DT, dt = qgwlib.check_timestep(p)
    assert DT == pytest.approx((4e6 / 255) ** 2 / (50 * 20), rel=1e-12)
    # biharmonic, beta-limited max has a < b false chain: DT_max = 1/(2 beta Lx)?  the
    # macro returns b = 0 whenever a < b; here a < 0 = b so DT_max = 1/0 = inf
    p2 = dict(C.cfg2(1024))
    p2.pop("dt")
    DT2, dt2 = qgwlib.check_timestep(p2)
    assert np.isinf(DT2)
    assert dt2 == pytest.approx(1.2078e4, rel=1e-3)


def test_topography_formula(qgwlib):
    p = dict(C.cfg1(32), h_topo=200.0, w_topo=3e5)
    nl, ny2, nx2 = 3, 33, 33
    topo = np.empty((ny2, nx2))
    lib = qgwlib.load()
    s = to_struct(p)
    assert lib.qgw_topo(ctypes.byref(s), topo.ctypes.data_as(ctypes.POINTER(ctypes.c_double))) == 0
    D = 4e6 / 32
    X = np.arange(nx2) * D
    Y = np.arange(ny2)[:, None] * D
    sh = lambda x, d: 1 - np.exp(-x ** 2 / (2 * d ** 2))
    ref = 200.0 * (1 - sh(X, 3e5) * sh(4e6 - X, 3e5) * sh(Y, 3e5) * sh(32 * D - Y, 3e5))
    assert np.allclose(topo, ref, rtol=1e-14, atol=1e-12)


@pytest.fixture(scope="module")
def dstcore(tmp_path_factory):
    so = str(tmp_path_factory.mktemp("dst") / "dstcore.so")
    # the work items move a buffer's values as floats, complex pairs and
    # 16-byte vectors; the device code separates those phases by warp or
    # block barriers, the loops here by nothing, hence no type-based aliasing
    subprocess.check_call(["g++", "-O2", "-fno-strict-aliasing", "-std=c++17", "-shared", "-fPIC", "-o", so,
                           os.path.join(ROOT, "tests", "cpu", "dst_core_check.cpp")])
    lib = ctypes.CDLL(so)
    lib.dst_core_run_f64.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
    lib.dst_core_run_f32.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
    lib.dst_warp_run_f32.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
    lib.dst_blue_run_f64.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
    lib.dst_blue_run_f32.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
    return lib


@pytest.mark.parametrize("M", [4, 8, 16, 32, 64, 128, 256, 512, 1024, 2048, 4096,
                               6, 10, 12, 14, 30, 42, 96, 100, 250, 384, 490, 1000, 1536, 2430])
def test_device_dst_blocks_on_host(dstcore, M):
    x = np.random.default_rng(M).standard_normal((3, M - 1))
    ref = sf.dst(x, type=1, axis=1)
    y = x.copy()
    dstcore.dst_core_run_f64(M, 3, y.ctypes.data)
    assert np.linalg.norm(y - ref) <= 1e-14 * np.linalg.norm(ref)
    yf = x.astype(np.float32)
    dstcore.dst_core_run_f32(M, 3, yf.ctypes.data)
    assert np.linalg.norm(yf - ref) <= 1e-5 * np.linalg.norm(ref)


@pytest.mark.parametrize("M", [512, 1024])
def test_warp_dst_on_host(dstcore, M):
    """The FP32 one-warp in-place transform (three DIF passes, digit-reversed
    split reads) with its lanes run in turn, against scipy's DST-I."""
    x = np.random.default_rng(M + 1).standard_normal((3, M - 1))
    ref = sf.dst(x, type=1, axis=1)
    yf = x.astype(np.float32)
    assert dstcore.dst_warp_run_f32(M, 3, yf.ctypes.data) == 1
    assert np.linalg.norm(yf - ref) <= 1e-5 * np.linalg.norm(ref)
    # a single impulse and a constant row
    for row in (np.eye(M - 1)[M // 3], np.ones(M - 1)):
        ref = sf.dst(row, type=1)
        yf = row.astype(np.float32).copy()
        assert dstcore.dst_warp_run_f32(M, 1, yf.ctypes.data) == 1
        assert np.linalg.norm(yf - ref) <= 1e-5 * np.linalg.norm(ref)


@pytest.mark.parametrize("M", [5, 9, 22, 23, 26, 99, 101, 998, 1001, 64, 1024])
def test_chirp_z_dst_on_host(dstcore, M):
    """The chirp-z (Bluestein) DST-I of lengths the half-length FFT cannot
    take (odd M; M/2 = 11, 13, 499) -- and of two it can, as a check of the
    form itself -- against scipy's DST-I."""
    x = np.random.default_rng(M + 7).standard_normal((3, M - 1))
    ref = sf.dst(x, type=1, axis=1)
    y = x.copy()
    dstcore.dst_blue_run_f64(M, 3, y.ctypes.data)
    assert np.linalg.norm(y - ref) <= 1e-14 * np.linalg.norm(ref), np.linalg.norm(y - ref) / np.linalg.norm(ref)
    yf = x.astype(np.float32)
    dstcore.dst_blue_run_f32(M, 3, yf.ctypes.data)
    assert np.linalg.norm(yf - ref) <= 2e-6 * np.linalg.norm(ref), np.linalg.norm(yf - ref) / np.linalg.norm(ref)


def test_supported_transform_lengths(dstcore):
    """Even lengths whose half factors into 2, 3, 5 and 7 take the half-length
    FFT; closed basins run the rest as chirp-z transforms, and the periodic
    basin refuses them (QGW_ERR_UNSUPPORTED at qgw_create)."""
    def smooth(n):
        for f in (2, 3, 5, 7):
            while n % f == 0:
                n //= f
        return n == 1
    for M in range(4, 4100):
        expect = M % 2 == 0 and smooth(M // 2)
        assert dstcore.dst_core_length_ok(M) == int(expect), M


@pytest.mark.parametrize("M", [16, 64, 128, 256, 512, 1024, 2048, 96, 1000])
def test_pass_ordered_twiddles(dstcore, M):
    """The Stockham passes' lane-ordered twiddle table holds w_H^(q k H/(Ns R))
    at (Ns - R0) + (q-1) Ns + k, H - R0 entries in all."""
    assert dstcore.dst_core_check_twp(M) == 0


@pytest.mark.parametrize("seed", [1, 7, 12345, 0])
def test_forcing_generator_is_the_c_library_rand(tmp_path, seed):
    """The stochastic forcing's generator restates the C library's rand()
    (the reference's noise source, src/forcing.h:62-63)."""
    so = str(tmp_path / "grand.so")
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-o", so,
                           os.path.join(ROOT, "tests", "cpu", "glibc_rand_check.cpp")])
    lib = ctypes.CDLL(so)
    lib.glibc_rand_mismatches.argtypes = [ctypes.c_uint, ctypes.c_int]
    assert lib.glibc_rand_mismatches(seed, 200000) == 0


def test_footprint_grows_with_size(qgwlib):
    small = qgwlib.footprint(C.cfg1(256), qgwlib.FP64)
    big = qgwlib.footprint(C.cfg2(1024), qgwlib.FP64)
    comp = qgwlib.footprint(C.cfg2(1024), qgwlib.FP32C)
    assert small < big and comp < big
    assert big > 7 * 10 * 1023 * 1024 * 8
