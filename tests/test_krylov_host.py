"""Host algebra of the Lanczos propagator (csrc/evr_krylov.h), compiled unchanged with g++
into a test harness: the Jacobi eigen-decomposition and u = exp(-i T t) e_1 against numpy
(1e-13 absolute)."""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "elvibrot-tnumtana_gb300", "csrc")

HARNESS = r"""
#include "evr_krylov.h"
extern "C" int eig(int n, double* A, double* w, double* V) {
  std::vector<double> a(A, A + (size_t)n * n), ww, vv;
  bool ok = evr::sym_eig_jacobi(n, a, ww, vv);
  for (int i = 0; i < n; ++i) w[i] = ww[i];
  for (size_t i = 0; i < (size_t)n * n; ++i) V[i] = vv[i];
  return ok ? 0 : 1;
}
extern "C" int ucol(int n, const double* a, const double* b, double t, double* ur, double* ui) {
  return evr::krylov_propagator_column(n, a, b, t, ur, ui) ? 0 : 1;
}
"""


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    if not shutil.which("g++"):
        pytest.skip("g++ not found")
    d = tmp_path_factory.mktemp("krylov")
    src, so = d / "h.cpp", d / "h.so"
    src.write_text(HARNESS)
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-I", CSRC, str(src), "-o", str(so)])
    L = C.CDLL(str(so))
    dp = C.POINTER(C.c_double)
    L.eig.argtypes = [C.c_int, dp, dp, dp]
    L.ucol.argtypes = [C.c_int, dp, dp, C.c_double, dp, dp]
    return L


def _p(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


@pytest.mark.parametrize("n", [1, 2, 7, 40])
def test_jacobi_eigendecomposition(lib, n):
    rng = np.random.default_rng(n)
    A = rng.standard_normal((n, n))
    A = np.asfortranarray(A + A.T)
    w, V = np.zeros(n), np.zeros((n, n), order="F")
    assert lib.eig(n, _p(A.copy(order="F")), _p(w), _p(V)) == 0
    assert np.allclose(np.sort(w), np.linalg.eigvalsh(A), atol=1e-12 * np.abs(A).max())
    assert np.abs(V.T @ V - np.eye(n)).max() < 1e-13
    assert np.abs(A @ V - V * w).max() < 1e-12 * np.abs(A).max()


@pytest.mark.parametrize("n,t", [(1, 3.0), (5, 0.7), (16, 40.0), (30, 2.5)])
def test_propagator_column_matches_expm(lib, n, t):
    import scipy.linalg as sla
    rng = np.random.default_rng(10 + n)
    a = rng.uniform(-0.05, 0.05, n)
    b = rng.uniform(0.0, 0.03, max(n - 1, 0))
    T = np.diag(a) + np.diag(b, 1) + np.diag(b, -1)
    ref = sla.expm(-1j * T * t)[:, 0]
    ur, ui = np.zeros(n), np.zeros(n)
    bb = b if n > 1 else np.zeros(1)
    assert lib.ucol(n, _p(a), _p(bb), t, _p(ur), _p(ui)) == 0
    assert np.abs(ur + 1j * ui - ref).max() < 1e-13
