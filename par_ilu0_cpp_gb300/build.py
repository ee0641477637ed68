"""In-tree build of the native libraries (nvcc, sm_103a only).

Produces, under par_ilu0_cpp_gb300/lib/:

* ``libpar-ilu0-gmres.so``   — the C++ API (lljbash::IluSolver, PreconditionedGmres),
  the CsrMatrix utilities, IlukSymbolic and all CUDA kernels.
* ``libpar-ilu0-gmres_c.so`` — the LLJBASH_* C ABI (include/ilu_solver_c.h, gmres_c.h,
  par_ilu0_gb300.h) on top of it.
* ``par-ilu0-benchmark`` — the command-line benchmark (the reference's test/benchmark.cpp
  options), over both libraries.

These are the two libraries the reference builds (src/CMakeLists.txt:11,
src_c/CMakeLists.txt:2), with the same names.  Translation units compile in parallel;
nothing here needs cmake.

    python -m par_ilu0_cpp_gb300.build
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
OBJ = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "lib")

CORE_LIB = "libpar-ilu0-gmres.so"
C_LIB = "libpar-ilu0-gmres_c.so"
BENCH_EXE = "par-ilu0-benchmark"  # the command-line benchmark (csrc/benchmark_main.cpp)

CORE_SOURCES = ["host_csr.cpp", "ilu_solver.cu", "gmres.cu", "mlp.cu", "batched.cu"]
C_SOURCES = ["c_api.cu"]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _cuda_lib_dir(nvcc: str) -> str:
    home = os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    for d in ("lib64", "lib", os.path.join("targets", "sbsa-linux", "lib"), os.path.join("targets", "x86_64-linux", "lib")):
        p = os.path.join(home, d)
        if os.path.exists(os.path.join(p, "libcudart.so")):
            return p
    return os.path.join(home, "lib64")


def _flags(debug: bool = False):
    f = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC,-fvisibility=default", "-I" + INCLUDE, "-I" + CSRC,
         "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills"]
    if debug:
        f += ["-DGB300_DEBUG"]
    return ARCH + f


def _compile(nvcc: str, src: str, debug: bool) -> str:
    os.makedirs(OBJ, exist_ok=True)
    out = os.path.join(OBJ, os.path.basename(src) + ".o")
    cmd = [nvcc, "-c", os.path.join(CSRC, src), "-o", out] + _flags(debug)
    if src.endswith(".cpp"):
        cmd += ["-x", "cu"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{res.stdout}\n{res.stderr}")
    return out


def build(debug: bool = False, verbose: bool = False) -> str:
    """Compiles both libraries; returns the lib directory."""
    nvcc = _nvcc()
    cudalib = _cuda_lib_dir(nvcc)
    sources = [s for s in CORE_SOURCES + C_SOURCES if os.path.exists(os.path.join(CSRC, s))]
    with cf.ThreadPoolExecutor(max_workers=min(8, len(sources))) as ex:
        objs = dict(zip(sources, ex.map(lambda s: _compile(nvcc, s, debug), sources)))
    os.makedirs(LIB, exist_ok=True)
    core = os.path.join(LIB, CORE_LIB)
    clib = os.path.join(LIB, C_LIB)
    link_common = ARCH + ["-shared", "-cudart", "shared", "-Xlinker", "-rpath=" + cudalib, "-L" + cudalib]
    core_objs = [objs[s] for s in CORE_SOURCES if s in objs]
    for out, ins, extra in ((core, core_objs, []),
                            (clib, [objs[s] for s in C_SOURCES],
                             ["-L" + LIB, "-l:" + CORE_LIB, "-Xlinker", "-rpath=$ORIGIN"])):
        tmp = out + ".tmp"
        cmd = [nvcc] + link_common + ins + extra + ["-o", tmp]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"link failed for {out}:\n{res.stdout}\n{res.stderr}")
        os.replace(tmp, out)
        if verbose:
            print("built", out, file=sys.stderr)
    # the command-line benchmark: host C++ over both libraries
    exe = os.path.join(LIB, BENCH_EXE)
    cxx = shutil.which(os.environ.get("CXX", "g++")) or "g++"
    cmd = [cxx, "-std=c++17", "-O2", "-I" + INCLUDE, os.path.join(CSRC, "benchmark_main.cpp"), "-o", exe + ".tmp",
           "-L" + LIB, "-l:" + C_LIB, "-l:" + CORE_LIB, "-Wl,-rpath,$ORIGIN"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"build failed for {BENCH_EXE}:\n{res.stdout}\n{res.stderr}")
    os.replace(exe + ".tmp", exe)
    return LIB


if __name__ == "__main__":
    build(debug="--debug" in sys.argv, verbose=True)
