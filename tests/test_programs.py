"""The drop-in boundary shown by a compiler: the reference's own C test programs
(test/test.c, test/amd_test.c) compiled UNCHANGED against this library's include/ and
linked with libpar-ilu0-gmres_c.so + libpar-ilu0-gmres.so (the reference's CMake links
the C library's users with both, src_c/CMakeLists.txt:4), and the command-line
benchmark par-ilu0-benchmark with the options of the reference's test/benchmark.cpp.

Compiling and linking run on the CPU; running the solver needs the GPU.  The reference
sources come from the checkout or the copy oracle/build_ref.sh stages in oracle/_ref."""
import os
import re
import shutil
import subprocess

import numpy as np
import pytest

import oracle
from conftest import ROOT
from par_ilu0_cpp_gb300 import api
from par_ilu0_cpp_gb300 import build as nb
from par_ilu0_cpp_gb300 import generators as g

LIB = os.path.join(ROOT, "par_ilu0_cpp_gb300", "lib")
BENCH = os.path.join(LIB, "par-ilu0-benchmark")


def _compile_reference_program(rel, out_dir):
    src = oracle.reference_file(rel)
    if src is None:
        pytest.skip(f"reference {rel} not available here")
    cc = shutil.which("gcc") or shutil.which("cc")
    exe = os.path.join(out_dir, os.path.basename(rel)[:-2])
    cmd = [cc, "-std=c99", "-O2", "-I" + os.path.join(ROOT, "include"), src, "-o", exe, "-L" + LIB,
           "-l:" + nb.C_LIB, "-l:" + nb.CORE_LIB, "-Wl,-rpath," + LIB, "-lm"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    return exe


def write_mm1(path, a):
    """1-based coordinate MatrixMarket file of a Csr."""
    rows = np.repeat(np.arange(a.n), np.diff(a.row_ptr))
    with open(path, "w") as fh:
        fh.write("%%MatrixMarket matrix coordinate real general\n")
        fh.write(f"{a.n} {a.n} {a.nnz}\n")
        for r, c, v in zip(rows, a.col_idx, a.values):
            fh.write(f"{int(r) + 1} {int(c) + 1} {float(v)!r}\n")


def _field(out, name):
    m = re.search(r"^" + re.escape(name) + r":\s+(\S+)", out, re.M)
    assert m, (name, out)
    return m.group(1)


def test_reference_c_programs_compile_and_link_unchanged(tmp_path):
    _compile_reference_program("test/test.c", str(tmp_path))
    _compile_reference_program("test/amd_test.c", str(tmp_path))


def test_benchmark_cli_usage():
    res = subprocess.run([BENCH, "--help"], capture_output=True, text=True)
    assert res.returncode == 0
    for flag in ("--mat", "--lof", "--amd", "--nd", "--eps", "--maxit", "--restart", "--threads", "--rep",
                 "--warmup", "--onlyfact", "--onlysubs"):
        assert flag in res.stdout
    bad = subprocess.run([BENCH, "--no-such-flag"], capture_output=True, text=True)
    assert bad.returncode != 0


@pytest.mark.gpu
def test_reference_test_c_runs(tmp_path):
    exe = _compile_reference_program("test/test.c", str(tmp_path))
    mm = str(tmp_path / "a.mtx")
    write_mm1(mm, g.convdiff3d(14))
    res = subprocess.run([exe, mm], capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stdout + res.stderr
    assert int(_field(res.stdout, "iter")) > 0
    assert float(_field(res.stdout, "max_err")) < 1e-6


@pytest.mark.gpu
@pytest.mark.parametrize("args", [[], ["-k", "1", "-r", "30"], ["--mixed"], ["-n", "2", "-w"], ["--warmup=2"]],
                         ids=["default", "ilu1_r30", "mixed", "rep2_warmup", "warmup2"])
def test_benchmark_cli_solves(tmp_path, args):
    a = g.laplace2d(48)
    mm = str(tmp_path / "a.mtx")
    write_mm1(mm, a)
    res = subprocess.run([BENCH, "-m", mm] + args, capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stdout + res.stderr
    out = res.stdout
    assert int(_field(out, "n")) == a.n and int(_field(out, "nnz")) == a.nnz
    assert float(_field(out, "max_err")) < 1e-5
    assert int(_field(out, "reps")) == (2 if "-n" in args else 1)
    its = [int(v) for v in re.findall(r"^iter: (\d+)", out, re.M)]
    assert its and len(set(its)) == 1  # every repetition takes the same iterations
    if not args or args == ["-k", "1", "-r", "30"]:
        # the library's own solve of the same system takes the same number of iterations
        lof = 1 if "-k" in args else 0
        m = 30 if "-r" in args else 60
        b = g.spmv(a, np.ones(a.n))
        res2, _, _ = api.ilu_gmres(a, b, lof=lof, tol=1e-8, restart=m, maxit=1000, relative=False)
        assert res2.iterations == its[0]


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["--onlyfact", "--onlysubs"])
def test_benchmark_cli_isolation_modes(tmp_path, mode):
    mm = str(tmp_path / "a.mtx")
    write_mm1(mm, g.convdiff3d(12))
    res = subprocess.run([BENCH, "-m", mm, mode, "-n", "3"], capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stdout + res.stderr
    assert "iter:" not in res.stdout
    if mode == "--onlyfact":
        assert float(_field(res.stdout, "total factorize time (s)")) > 0
    else:
        assert float(_field(res.stdout, "total precon time (s)")) > 0


def test_reference_amd_test_runs_on_the_host(tmp_path):
    """The reference's test/amd_test.c (unchanged) prints the pattern of a 5x5 matrix in
    its AMD order; CsrAmdOrder returns 0 and a permutation."""
    exe = _compile_reference_program("test/amd_test.c", str(tmp_path))
    res = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert res.returncode == 0, res.stdout + res.stderr
    assert "ret: 0" in res.stdout
    perm = re.search(r"P:\n((?: \d+)+)", res.stdout).group(1).split()
    assert sorted(int(v) for v in perm) == list(range(5))


@pytest.mark.gpu
@pytest.mark.parametrize("flag", ["--amd", "--nd"])
def test_benchmark_cli_reordered(tmp_path, flag):
    mm = str(tmp_path / "a.mtx")
    write_mm1(mm, g.convdiff3d(16))
    res = subprocess.run([BENCH, "-m", mm, flag, "-k", "1"], capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stdout + res.stderr
    assert float(_field(res.stdout, "max_err")) < 1e-5
    assert int(_field(res.stdout, "iter")) > 0
