"""Host-side check of the sparse pre-elimination planner (no GPU): the planned
levels plus a dense LU of the remaining core give the full matrix's log|det| and
solution (gpusgdlm_gb300/csrc/elimination.cu, evaluated in FP64)."""
import ctypes as C
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def elim(tmp_path_factory):
    out = tmp_path_factory.mktemp("elim") / "libelim_check.so"
    cuda_inc = "/usr/local/cuda/include"
    r = subprocess.run(["g++", "-O1", "-std=c++17", "-shared", "-fPIC", "-x", "c++",
                        str(ROOT / "tests" / "elim_check.cpp"), "-I", cuda_inc, "-o", str(out)],
                       capture_output=True, text=True)
    if r.returncode != 0:
        pytest.skip("cannot build the planner harness: " + r.stderr[:300])
    L = C.CDLL(str(out))
    L.elim_check.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p,
                             C.c_void_p, C.c_void_p]
    return L


def run(L, sp, theta_e, levels, rhs):
    P, m = sp.shape
    spu = np.asfortranarray(sp.astype(np.uint32))
    th = np.ascontiguousarray(theta_e, dtype=np.float64)
    sol = np.zeros(m); info = np.zeros(4)
    L.elim_check(m, P, spu.ctypes.data, th.ctypes.data, levels, rhs.ctypes.data, sol.ctypes.data,
                 info.ctypes.data)
    return info, sol


def full_matrix(sp, theta_e):
    P, m = sp.shape
    A = np.eye(m)
    for j in range(m):
        for k in range(P):
            pos = int(sp[k, j])
            if pos < m * m:
                A[pos % m, pos // m] = -theta_e[j * P + k]
    return A


@pytest.mark.parametrize("m,kmax,seed", [(6, 3, 0), (40, 6, 1), (400, 17, 2)])
@pytest.mark.parametrize("levels", [0, 1, 3])
def test_plan_reproduces_dense_logdet_and_solve(elim, m, kmax, seed, levels):
    rng = np.random.default_rng(seed)
    P = 3 + kmax
    sp = np.full((P, m), 2147483648, dtype=np.uint64)
    for j in range(m):
        k = int(rng.integers(0, kmax + 1))
        pars = rng.choice(np.delete(np.arange(m), j), size=min(k, m - 1), replace=False)
        for t, par in enumerate(pars):
            sp[3 + t, j] = j + m * par
    theta = rng.normal(0, 0.1, m * P)
    rhs = rng.normal(0, 1, m)
    info, sol = run(elim, sp, theta, levels, rhs)
    A = full_matrix(sp, theta)
    sign, ld = np.linalg.slogdet(A)
    assert info[1] >= 1  # -1: a solve program reads a slot outside the solve prefix
    np.testing.assert_allclose(info[0], ld, rtol=1e-10, atol=1e-11)
    np.testing.assert_allclose(sol, np.linalg.solve(A, rhs), rtol=1e-9, atol=1e-11)
    if levels == 0:
        assert info[1] == m and info[2] == 0
    if m == 400 and levels == 3:
        assert info[1] <= 300  # the dense core shrinks substantially


def test_graph_without_edges_keeps_one_core_node(elim):
    m, P = 50, 3
    sp = np.full((P, m), 2147483648, dtype=np.uint64)
    info, sol = run(elim, sp, np.zeros(m * P), 3, np.arange(m, dtype=float))
    assert info[1] == 1 and info[0] == 0.0
    np.testing.assert_allclose(sol, np.arange(m))
