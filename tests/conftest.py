"""Shared fixtures.  GPU tests are marked ``gpu`` and call the native library through
the C ABI; everything else runs on the CPU (oracle, host logic, ABI loading)."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden", "golden_cases.npz")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built native library")


def _gpu_available() -> bool:
    """True when the machine has a CUDA GPU.  The native library is NOT consulted: on a
    GPU machine a missing or broken library makes the gpu tests fail, never skip."""
    import shutil
    import subprocess

    if shutil.which("nvidia-smi") is None:
        return False
    try:
        out = subprocess.run(["nvidia-smi", "-L"], capture_output=True, text=True, timeout=60)
    except Exception:
        return False
    return out.returncode == 0 and "GPU" in out.stdout


def pytest_collection_modifyitems(config, items):
    if _gpu_available():
        return
    skip = pytest.mark.skip(reason="no CUDA GPU available")
    for item in items:
        if "gpu" in item.keywords:
            item.add_marker(skip)


class GoldenCase:
    def __init__(self, data, name):
        from par_ilu0_cpp_gb300.generators import Csr

        self.name = name
        g = lambda k: data[name + "/" + k]  # noqa: E731
        self.a = Csr(len(g("a_rp")) - 1, g("a_rp"), g("a_ci"), g("a_val"))
        self.lof = int(g("lof"))
        self.restart = int(g("restart"))
        self.f_rp = g("f_rp")
        self.f_ci = g("f_ci")
        self.nzmap = g("nzmap")
        self.diag = g("diag")
        self.etree_l = g("etree_l")
        self.etree_u = g("etree_u")
        self.level_l = g("level_l")
        self.level_u = g("level_u")
        self.nlev = g("nlev")
        self.lu = g("lu")
        self.x_true = g("x_true")
        self.b = g("b")
        self.x_subs = g("x_subs")
        self.tol = float(g("tol"))
        self.gmres_ok = bool(g("gmres_ok"))
        self.gmres_iters = int(g("gmres_iters"))
        self.gmres_x = g("gmres_x")

    def f_csr(self):
        """F pattern with A's values scattered (fill = 0), as test/benchmark.cpp:116-119."""
        from par_ilu0_cpp_gb300.generators import Csr

        v = np.zeros(len(self.f_ci))
        v[self.nzmap] = self.a.values
        return Csr(self.a.n, self.f_rp, self.f_ci, v)


def _load_golden():
    data = np.load(GOLDEN)
    return [GoldenCase(data, str(n)) for n in data["names"]]


GOLDEN_CASES = _load_golden()


@pytest.fixture(params=GOLDEN_CASES, ids=lambda c: c.name)
def golden(request):
    return request.param


def rel_err(x, ref, floor=None):
    """max |x - ref| / max(|ref|, floor) with floor = 1e-3 * max|ref| by default (mixed
    absolute/relative criterion for entries near zero)."""
    x = np.asarray(x, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    if ref.size == 0:
        return 0.0
    if floor is None:
        floor = 1e-3 * float(np.max(np.abs(ref))) if np.any(ref) else 1.0
    return float(np.max(np.abs(x - ref) / np.maximum(np.abs(ref), floor)))


# ---- matrix builders shared by the GPU parity tests and the oracle tests ----
def csr_from_rows(n, cols_of_row, vals_of_row):
    """Csr from per-row column and value lists (columns ascending)."""
    from par_ilu0_cpp_gb300 import generators as g

    rp = np.zeros(n + 1, dtype=np.int64)
    for i in range(n):
        rp[i + 1] = rp[i] + len(cols_of_row[i])
    ci = np.concatenate([np.asarray(c, dtype=np.int64) for c in cols_of_row]) if n else np.zeros(0, np.int64)
    va = np.concatenate([np.asarray(v, dtype=np.float64) for v in vals_of_row]) if n else np.zeros(0)
    return g.Csr(n, rp, ci, va)


def banded(n, w, seed):
    """Diagonally dominant matrix with full bandwidth w on both sides: rows of up to w
    entries per triangle, a dependency chain of n levels."""
    from par_ilu0_cpp_gb300 import generators as g

    rng = np.random.default_rng(seed)
    rows, cols = [], []
    for i in range(n):
        c = np.arange(max(0, i - w), min(n, i + w + 1))
        rows.append(np.full(c.size, i))
        cols.append(c)
    r = np.concatenate(rows)
    c = np.concatenate(cols)
    v = rng.uniform(-1.0, 1.0, r.size)
    v[r == c] = 2.0 * w + 2.0
    rp = np.zeros(n + 1, dtype=np.int64)
    np.add.at(rp, r + 1, 1)
    return g.Csr(n, np.cumsum(rp), c, v)


def ragged(n, kmax, seed):
    """Non-symmetric pattern, rows with 0 .. kmax off-diagonal entries at random columns,
    diagonally dominant values."""
    rng = np.random.default_rng(seed)
    cols, vals = [], []
    for i in range(n):
        k = int(rng.integers(0, kmax + 1))
        c = np.unique(rng.integers(0, n, size=k))
        c = c[c != i]
        v = rng.uniform(-1.0, 1.0, size=c.size)
        cc = np.append(c, i)
        vv = np.append(v, np.abs(v).sum() + 1.0)
        o = np.argsort(cc)
        cols.append(cc[o])
        vals.append(vv[o])
    return csr_from_rows(n, cols, vals)
