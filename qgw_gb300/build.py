"""Build libqgw_gpu.so in-tree (qgw_gb300/lib/) with nvcc for sm_103a.

Translation units are compiled in parallel; the link uses nvcc's static
CUDA runtime so the library does not depend on a loader path for cudart.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "lib")
LIB = os.path.join(OUT, "libqgw_gpu.so")
DRIVER = os.path.join(OUT, "qg_gpu")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# -fmad=false: no implicit multiply-add contraction.  Every FMA of the hot
# loops is explicit (fmaT), so an expression rounds the same way in every
# kernel it is inlined into (a run gives bitwise the same result alone and in
# an ensemble), and the scalar dt/AB3 formulas round like the reference's.
NVFLAGS = ["-O3", "-std=c++17", "-lineinfo", "-fmad=false", "-Xcompiler", "-fPIC,-O2",
           "--expt-relaxed-constexpr"] + ARCH
CXXFLAGS = ["-O2", "-std=c++17", "-fPIC", "-Wall", "-Wno-unknown-pragmas", "-pthread"]


def cuda_include() -> str:
    return os.path.join(os.path.dirname(os.path.dirname(nvcc())), "include")

CU_SOURCES = ["kernels.cu", "kernels_f32c.cu", "kernels_ens.cu", "kernels_ens_f32c.cu", "api.cu", "ensemble.cu", "probe.cu",
              "noalloc.cu"]
CXX_SOURCES = ["host.cpp", "ncio.cpp", "serve.cpp"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _sources():
    cu = [s for s in CU_SOURCES if os.path.exists(os.path.join(SRC, s))]
    return cu, CXX_SOURCES


def _stale(objs, srcs) -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(SRC, f) for f in os.listdir(SRC)]
    deps += [os.path.join(HERE, "driver", f) for f in os.listdir(os.path.join(HERE, "driver"))]
    deps.append(os.path.join(HERE, "..", "include", "qgw_gpu.h"))
    deps.append(os.path.abspath(__file__))
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(verbose: bool = False, force: bool = False, ptxas_v: bool = False) -> str:
    cu, cxx = _sources()
    objdir = os.path.join(OUT, "obj")
    os.makedirs(objdir, exist_ok=True)
    if not force and not _stale(None, None):
        return LIB
    nv = nvcc()
    jobs = []
    for s in cu:
        o = os.path.join(objdir, s + ".o")
        flags = NVFLAGS + (["-Xptxas", "-v"] if ptxas_v else [])
        jobs.append((s, [nv] + flags + ["-c", os.path.join(SRC, s), "-o", o], o))
    for s in cxx:
        o = os.path.join(objdir, s + ".o")
        jobs.append((s, ["g++"] + CXXFLAGS + ["-I", cuda_include(), "-c", os.path.join(SRC, s), "-o", o], o))

    def run(job):
        name, cmd, _ = job
        res = subprocess.run(cmd, capture_output=True, text=True)
        return name, cmd, res

    with cf.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
        results = list(ex.map(run, jobs))
    for name, cmd, res in results:
        if verbose or ptxas_v:
            sys.stderr.write(res.stderr)
        if res.returncode != 0:
            raise RuntimeError(f"compiling {name} failed:\n{' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    objs = [j[2] for j in jobs]
    tmp = LIB + ".tmp"
    link = [nv] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart_static", "-ldl", "-lrt", "-lpthread"]
    res = subprocess.run(link, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{' '.join(link)}\n{res.stderr}")
    os.replace(tmp, LIB)
    # the qg executable on top of the library (rpath: same directory)
    drv = [("g++", os.path.join(HERE, "driver", "qg_gpu.cpp"), DRIVER)]
    for cxx, src, out in drv:
        cmd = [cxx] + CXXFLAGS + [src, "-o", out + ".tmp", "-L", OUT, "-lqgw_gpu", "-Wl,-rpath,$ORIGIN", "-lm"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"building {out} failed:\n{' '.join(cmd)}\n{res.stderr}")
        os.replace(out + ".tmp", out)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv, ptxas_v="-v" in sys.argv))
