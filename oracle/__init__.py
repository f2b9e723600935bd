"""CPU oracle for the SGDLM hot path -- TEST INFRASTRUCTURE ONLY.

A plain C++ FP64 restatement of the reference algorithm (lutzgruber/gpuSGDLM,
rSGDLM/src/SGDLM/SGDLM.cu and rSGDLM/src/kernel_functions.cuh), loaded through
ctypes.  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg
may import this package; the product (gpusgdlm_gb300) never does.

Parity pin: oracle/ref_driver.cpp compiles the reference's own kernel header for
the CPU (oracle/build_ref.sh, outputs in oracle/_ref/) and tests/golden/
make_golden.py records its outputs; tests/test_oracle_golden.py checks this
oracle against those fixtures.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "libsgdlm_oracle.so"
SRC = HERE / "sgdlm_oracle.cpp"


def build(force: bool = False) -> Path:
    """g++ -O2 -fopenmp; no fast-math, so the oracle keeps IEEE FP64 semantics."""
    if force or not LIB.exists() or LIB.stat().st_mtime < SRC.stat().st_mtime:
        cmd = ["g++", "-O2", "-std=c++17", "-fopenmp", "-fPIC", "-shared", str(SRC), "-o", str(LIB)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("oracle build failed:\n" + r.stderr)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(LIB))
        d, i, u32, u64, l = C.c_double, C.c_int, C.c_uint32, C.c_uint64, C.c_long
        P_d, P_u = C.POINTER(C.c_double), C.POINTER(C.c_uint)
        L.orc_philox.argtypes = [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]
        L.orc_psi.argtypes = [d]; L.orc_psi.restype = d
        L.orc_psi1.argtypes = [d]; L.orc_psi1.restype = d
        L.orc_mt_try.argtypes = [d, d, d]; L.orc_mt_try.restype = d
        L.orc_posterior.argtypes = [i, i, P_u, P_d, P_d, P_d, P_d, P_d, P_d]
        L.orc_prior.argtypes = [i, i, P_u, P_d, P_d, P_d, P_d, P_d]
        L.orc_cholesky.argtypes = [i, i, P_u, P_d, P_d]
        L.orc_sample.argtypes = [i, i, P_u, P_d, P_d, P_d, P_d, l, u64, u64, P_d, P_d, i]
        L.orc_sample.restype = l
        L.orc_logdet.argtypes = [i, i, P_u, l, P_d, P_d, i]
        L.orc_weights.argtypes = [l, P_d, P_d]; L.orc_weights.restype = d
        L.orc_vb.argtypes = [i, i, P_u, P_d, P_d, l, P_d, P_d, P_d, P_d, P_d, P_d, P_d, P_d]
        L.orc_forecast.argtypes = [i, i, P_u, l, P_d, P_d, P_d, u64, u64, P_d, P_d, i]
        L.orc_evolve.argtypes = [i, i, P_u, P_d, P_d, P_d, P_d, P_d, l, u64, u64, C.c_uint, P_d,
                                 P_d, i]
        L.orc_evo_prior.argtypes = [i, i, P_u, P_d, P_d, P_d, P_d, P_d, P_d, P_d]
        L.orc_evolve.restype = l
        _lib = L
    return _lib


def _d(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _u(a):
    return a.ctypes.data_as(C.POINTER(C.c_uint))


def f64(a):
    return np.asfortranarray(np.asarray(a, dtype=np.float64)).copy(order="F")


def u32(a):
    return np.asfortranarray(np.asarray(a, dtype=np.uint32)).copy(order="F")


def philox(ctr, key):
    c = (C.c_uint32 * 4)(*ctr); k = (C.c_uint32 * 2)(*key); o = (C.c_uint32 * 4)()
    lib().orc_philox(c, k, o)
    return list(o)


def psi(x):
    return lib().orc_psi(float(x))


def psi1(x):
    return lib().orc_psi1(float(x))


def mt_try(alpha, x, u):
    return lib().orc_mt_try(float(alpha), float(x), float(u))


def posterior(p, m_t, C_t, n_t, s_t, y, F):
    """Returns updated copies (m, C, n, s)."""
    P, m = m_t.shape
    p, m_t, C_t, n_t, s_t, y, F = u32(p), f64(m_t), f64(C_t), f64(n_t), f64(s_t), f64(y), f64(F)
    lib().orc_posterior(m, P, _u(p), _d(m_t), _d(C_t), _d(n_t), _d(s_t), _d(y), _d(F))
    return m_t, C_t, n_t, s_t


def prior(p, C_t, n_t, beta, delta, W_t=None):
    P, _, m = C_t.shape
    p, C_t, n_t, beta, delta = u32(p), f64(C_t), f64(n_t), f64(beta), f64(delta)
    W_t = f64(np.zeros_like(C_t) if W_t is None else W_t)
    lib().orc_prior(m, P, _u(p), _d(C_t), _d(n_t), _d(W_t), _d(beta), _d(delta))
    return C_t, n_t, W_t


def cholesky(p, C_t):
    P, _, m = C_t.shape
    p, C_t = u32(p), f64(C_t)
    U = np.zeros_like(C_t, order="F")
    lib().orc_cholesky(m, P, _u(p), _d(C_t), _d(U))
    return U


def sample(p, m_t, C_t, n_t, s_t, n, seed, epoch, nthreads=0):
    """Series-major draws: lambda (n, m) Fortran = [j*n + i], theta (P, n, m) Fortran."""
    P, m = m_t.shape
    p, m_t, C_t, n_t, s_t = u32(p), f64(m_t), f64(C_t), f64(n_t), f64(s_t)
    lam = np.zeros((n, m), order="F"); th = np.zeros((P, n, m), order="F")
    capped = lib().orc_sample(m, P, _u(p), _d(m_t), _d(C_t), _d(n_t), _d(s_t), n, seed, epoch,
                              _d(lam), _d(th), nthreads)
    return lam, th, capped


def logdet(sp, theta, nthreads=0):
    P, n, m = theta.shape
    sp, theta = u32(sp), f64(theta)
    out = np.zeros(n)
    lib().orc_logdet(m, P, _u(sp), n, _d(theta), _d(out), nthreads)
    return out


def weights(ld):
    ld = f64(ld); w = np.zeros_like(ld)
    s = lib().orc_weights(len(ld), _d(ld), _d(w))
    return w, s


def vb(p, n_t, s_t, w, lam, theta):
    P, n, m = theta.shape
    p, n_t, s_t, w, lam, theta = u32(p), f64(n_t), f64(s_t), f64(w), f64(lam), f64(theta)
    mm = np.zeros((P, m), order="F"); Cm = np.zeros((P, P, m), order="F")
    nm = np.zeros(m); sm = np.zeros(m); aux = np.zeros((3, m), order="F")
    lib().orc_vb(m, P, _u(p), _d(n_t), _d(s_t), n, _d(w), _d(lam), _d(theta), _d(mm), _d(Cm),
                 _d(nm), _d(sm), _d(aux))
    return dict(m=mm, C=Cm, n=nm, s=sm, mean_lambda=aux[0], mean_log_lambda=aux[1], mean_Q=aux[2])


def forecast(sp, lam, theta, x, seed, epoch, nthreads=0):
    """Returns y (m, n) Fortran == reference layout, and the per-draw log|det|."""
    P, n, m = theta.shape
    sp, lam, theta, x = u32(sp), f64(lam), f64(theta), f64(x)
    y = np.zeros((m, n), order="F"); ld = np.zeros(n)
    lib().orc_forecast(m, P, _u(sp), n, _d(lam), _d(theta), _d(x), seed, epoch, _d(y), _d(ld), nthreads)
    return y, ld


def evolve(p, W_t, r_t, c_t, beta, lam, theta, seed, epoch, compat, nthreads=0, G=None):
    P, n, m = theta.shape
    p, W_t, r_t, c_t, beta = u32(p), f64(W_t), f64(r_t), f64(c_t), f64(beta)
    lam, theta = f64(lam), f64(theta)
    Gp = None if G is None else f64(G)
    capped = lib().orc_evolve(m, P, _u(p), _d(W_t), _d(r_t), _d(c_t), _d(beta),
                              None if Gp is None else _d(Gp), n, seed, epoch, compat, _d(lam),
                              _d(theta), nthreads)
    return lam, theta, capped


def evo_prior(p, m_t, C_t, n_t, beta, delta, G):
    """compute_one_step_ahead_prior with an evolution matrix: (a, R, r, W)."""
    P, _, m = C_t.shape
    p, m_t, C_t, n_t = u32(p), f64(m_t), f64(C_t), f64(n_t)
    beta, delta, G = f64(beta), f64(delta), f64(G)
    W_t = f64(np.zeros_like(C_t))
    lib().orc_evo_prior(m, P, _u(p), _d(m_t), _d(C_t), _d(n_t), _d(W_t), _d(beta), _d(delta),
                        _d(G))
    return m_t, C_t, n_t, W_t
