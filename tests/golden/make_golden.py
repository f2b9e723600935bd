"""Generates tests/golden/*.npz from the reference's own kernels run on the CPU.

Run with the reference checkout:  python tests/golden/make_golden.py <reference checkout>
(or SGDLM_REFERENCE=<checkout>).  It builds oracle/_ref/libref_kernels.so with oracle/build_ref.sh, feeds the
reference's kernels (rSGDLM/src/kernel_functions.cuh, launched with the
shapes of rSGDLM/src/SGDLM/SGDLM.cu) seeded inputs, and stores inputs and outputs.
Where the reference consumes cuRAND output, the inputs are the GB300 library's
Philox normals for a recorded (seed, epoch), regenerated here in Python, so the
fixtures pin both the oracle and the device path draw by draw.
The reference (lutzgruber/gpuSGDLM) ships no tests or fixtures of its own.
"""
from __future__ import annotations

import ctypes as C
import math
import subprocess
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
import oracle  # noqa: E402  (test infrastructure)

OUT = Path(__file__).resolve().parent
NA = 2147483648  # R's NA_integer_ read as unsigned (memory_manager_RCPP.hpp:31-45)
TAG_THETA, TAG_NU, TAG_OMEGA = 2, 3, 6


def reference_checkout():
    import os

    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("SGDLM_REFERENCE")
    if not ref:
        sys.exit("usage: make_golden.py <reference checkout> (or set SGDLM_REFERENCE)")
    return ref


def ref_lib():
    subprocess.run([str(ROOT / "oracle" / "build_ref.sh"), reference_checkout()], check=True,
                   capture_output=True)
    L = C.CDLL(str(ROOT / "oracle" / "_ref" / "libref_kernels.so"))
    d, i, l = C.c_double, C.c_int, C.c_long
    Pd, Pu = C.POINTER(C.c_double), C.POINTER(C.c_uint)
    L.ref_psi.argtypes = [d]; L.ref_psi.restype = d
    L.ref_psi1.argtypes = [d]; L.ref_psi1.restype = d
    L.ref_posterior.argtypes = [i, i, Pu, Pd, Pd, Pd, Pd, Pd, Pd]
    L.ref_prior.argtypes = [i, i, Pu, Pd, Pd, Pd, Pd, Pd]
    L.ref_cholesky.argtypes = [i, i, Pu, Pd, Pd]
    L.ref_thetas.argtypes = [i, i, Pu, Pd, Pd, Pd, l, Pd, Pd, Pd]
    L.ref_make_gamma2.argtypes = [i, l, i, Pd, Pd, Pd, Pd, Pd]
    L.ref_make_beta.argtypes = [i, l, i, Pd, Pd, Pd, Pd, Pd]
    L.ref_vb.argtypes = [i, i, Pu, Pu, Pd, Pd, l, Pd, Pd, Pd, Pd, Pd, Pd, Pd, Pd, Pd]
    L.ref_forecast.argtypes = [i, i, Pu, l, Pd, Pd, Pd, Pd, Pd]
    L.ref_evolve_theta.argtypes = [i, i, Pu, Pd, Pd, l, Pd, Pd, Pd]
    L.ref_evo_prior.argtypes = [i, i, Pu, Pd, Pd, Pd, Pd, Pd, Pd, Pd]
    L.ref_evolve_theta_g.argtypes = [i, i, Pu, Pd, Pd, l, Pd, Pd, Pd, Pd]
    return L


def D(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def U(a):
    return a.ctypes.data_as(C.POINTER(C.c_uint))


def f64(a):
    return np.asfortranarray(np.array(a, dtype=np.float64))


def philox_normals(seed, epoch, tag, n, m, count):
    """Draw-major (n, m, count) standard normals of the library's stream."""
    k0, k1 = seed & 0xFFFFFFFF, seed >> 32
    z = np.zeros((n, m, count))
    for i in range(n):
        for j in range(m):
            for q in range((count + 3) // 4):
                r = oracle.philox((i, j, (tag << 24) | q, epoch & 0xFFFFFFFF), (k0, k1))
                vals = []
                for a, b in ((r[0], r[1]), (r[2], r[3])):
                    u1 = (a + 0.5) * 2.3283064365386963e-10
                    u2 = (b + 0.5) * 2.3283064365386963e-10
                    rad = math.sqrt(-2.0 * math.log(u1))
                    ang = 2.0 * math.pi * u2
                    vals += [rad * math.cos(ang), rad * math.sin(ang)]
                for t in range(4):
                    if 4 * q + t < count:
                        z[i, j, 4 * q + t] = vals[t]
    return z


def readme_parents():
    """The README scenario (README.md:48-73): m = 6, max p = 5."""
    m = 6
    count = [2, 0, 1, 3, 1, 2]
    sim = [[6], [1, 6, 4], [], [1, 2], [], [2, 4]]
    p = [c + len(s) for c, s in zip(count, sim)]
    P = max(p)
    sp = np.full((P, m), NA, dtype=np.uint32)
    for j in range(m):
        for t, par in enumerate(sim[j]):
            sp[count[j] + t, j] = j + m * (par - 1)  # helper_pos_Gamma[j, parent]
    return np.array(p, dtype=np.uint32), np.asfortranarray(sp)


def random_parents(rng, m, n_ext, kmax):
    ks = rng.integers(0, kmax + 1, size=m)
    p = n_ext + ks
    P = int(p.max())
    sp = np.full((P, m), NA, dtype=np.uint32)
    for j in range(m):
        others = [q for q in range(m) if q != j]
        pars = rng.choice(others, size=ks[j], replace=False)
        for t, par in enumerate(pars):
            sp[n_ext + t, j] = j + m * par
    return p.astype(np.uint32), np.asfortranarray(sp)


def random_state(rng, m, P, p, off_block=True):
    m_t = f64(rng.normal(0, 0.2, (P, m)))
    C_t = np.zeros((P, P, m), order="F")
    for j in range(m):
        A = rng.normal(0, 0.3, (P, P))
        S = A @ A.T / P + 0.05 * np.eye(P)
        if not off_block:
            S[p[j]:, :] = 0
            S[:, p[j]:] = 0
        C_t[:, :, j] = S
    n_t = f64(rng.uniform(3, 30, m))
    s_t = f64(rng.uniform(0.001, 0.01, m))
    return m_t, C_t, n_t, s_t


def case_posterior_prior(L, rng, name, p, sp):
    P, m = sp.shape
    m_t, C_t, n_t, s_t = random_state(rng, m, P, p, off_block=True)
    y = f64(rng.normal(0.1, 0.05, m))
    F = np.zeros((P, m), order="F")
    for j in range(m):
        F[: p[j], j] = rng.normal(0, 1, p[j])
    inputs = dict(p=p, sp=sp, m_t=m_t.copy(order="F"), C_t=C_t.copy(order="F"), n_t=n_t.copy(),
                  s_t=s_t.copy(), y=y, F=F)
    pm, pC, pn, ps = m_t.copy(order="F"), C_t.copy(order="F"), n_t.copy(), s_t.copy()
    L.ref_posterior(m, P, U(p), D(pm), D(pC), D(pn), D(ps), D(y), D(F))
    beta = f64(rng.uniform(0.9, 0.99, m))
    delta = np.asfortranarray(rng.uniform(0.9, 0.999, (P, P, m)))
    rC, rn = pC.copy(order="F"), pn.copy()
    W = np.zeros((P, P, m), order="F")
    L.ref_prior(m, P, U(p), D(rC), D(rn), D(W), D(beta), D(delta))
    U_ = np.zeros((P, P, m), order="F")
    L.ref_cholesky(m, P, U(p), D(pC), D(U_))
    np.savez(OUT / f"{name}_posterior_prior.npz", **inputs, post_m=pm, post_C=pC, post_n=pn,
             post_s=ps, beta=beta, delta=delta, prior_C=rC, prior_n=rn, prior_W=W, chol_post_C=U_)


def case_sampling_vb_forecast(L, rng, name, p, sp, n, seed, epoch):
    """VB on the oracle's draws of a valid posterior; forecast; evolve."""
    P, m = sp.shape
    m_t, C_t, n_t, s_t = random_state(rng, m, P, p, off_block=False)
    for j in range(m):
        m_t[p[j]:, j] = 0.0
    # gamma shapes >= 1 so the reference's sampler would not skip any series
    lam_o, th_o, capped = oracle.sample(p, m_t, C_t, n_t, s_t, n, seed, epoch)
    assert capped == 0
    # draw-major copies for the reference kernels
    lam_dm = np.ascontiguousarray(lam_o)              # (n, m) C-order == [i*m + j]
    th_dm = np.ascontiguousarray(th_o.transpose(1, 2, 0))  # (n, m, P) C-order
    z = philox_normals(seed, epoch, TAG_THETA, n, m, P)
    th_ref = np.zeros_like(th_dm)
    L.ref_thetas(m, P, U(p), D(m_t), D(C_t), D(s_t), n, D(lam_dm), D(np.ascontiguousarray(z)),
                 D(th_ref))
    # VB
    w = np.zeros(n); sw = np.zeros(1)
    mm = np.zeros((P, m), order="F"); Cm = np.zeros((P, P, m), order="F")
    nm = np.zeros(m); smn = np.zeros(m); aux = np.zeros(3 * m)
    th_work = th_dm.copy()
    L.ref_vb(m, P, U(p), U(sp), D(n_t), D(s_t), n, D(lam_dm), D(th_work), D(w), D(sw), D(mm),
             D(Cm), D(nm), D(smn), D(aux))
    # forecast from the same draws
    x = np.zeros((P, m), order="F")
    for j in range(m):
        for k in range(P):
            if sp[k, j] >= m * m and k < p[j]:
                x[k, j] = rng.normal(0, 1)
    nus = philox_normals(seed, epoch, TAG_NU, n, m, 1)[:, :, 0]
    y = np.zeros((n, m))
    L.ref_forecast(m, P, U(sp), n, D(lam_dm), D(th_dm), D(x), D(np.ascontiguousarray(nus)), D(y))
    # evolve: theta update with the reference's scale_omegas geometry
    W = np.zeros((P, P, m), order="F")
    for j in range(m):
        A = rng.normal(0, 0.05, (p[j], p[j]))
        W[: p[j], : p[j], j] = A @ A.T + 1e-4 * np.eye(p[j])
    c_t = f64(rng.uniform(0.002, 0.02, m))
    r_t = f64(rng.uniform(8, 20, m))
    beta = f64(np.full(m, 0.95)); beta[0] = 1.0
    ev_epoch = epoch + 1
    lam_ev, th_ev_o, capped = oracle.evolve(p, W, r_t, c_t, beta, lam_o, th_o, seed, ev_epoch, compat=3)
    om = philox_normals(seed, ev_epoch, TAG_OMEGA, n, m, P)
    th_ev_ref = th_dm.copy()
    L.ref_evolve_theta(m, P, U(p), D(W), D(c_t), n, D(np.ascontiguousarray(lam_ev)),
                       D(np.ascontiguousarray(om)), D(th_ev_ref))
    np.savez(OUT / f"{name}_vb_forecast.npz", p=p, sp=sp, m_t=m_t, C_t=C_t, n_t=n_t, s_t=s_t,
             n=n, seed=seed, epoch=epoch, lambdas=lam_dm, thetas_ref=th_ref, w=w, sum_w=sw[0],
             vb_m=mm, vb_C=Cm, vb_n=nm, vb_s=smn, vb_aux=aux.reshape(3, m), x=x, y_ref=y,
             W=W, c_t=c_t, r_t=r_t, beta=beta, ev_epoch=ev_epoch, lambdas_ev=np.ascontiguousarray(lam_ev),
             thetas_ev_ref=th_ev_ref)


def case_evolution_matrix(L, rng, name, p, sp, n, seed, epoch):
    """computeEvoPrior (a = G m, R = G R G' with the reference's cut-offs) and the
    evolution of forecast draws with G (theta = G theta + chol(W)' omega)."""
    P, m = sp.shape
    m_t, C_t, n_t, s_t = random_state(rng, m, P, p, off_block=True)
    beta = f64(rng.uniform(0.9, 0.99, m))
    delta = np.asfortranarray(rng.uniform(0.9, 0.999, (P, P, m)))
    G = np.asfortranarray(np.repeat(np.eye(P)[:, :, None], m, axis=2) + rng.normal(0, 0.1, (P, P, m)))
    a, R, r = m_t.copy(order="F"), C_t.copy(order="F"), n_t.copy()
    W = np.zeros((P, P, m), order="F")
    L.ref_evo_prior(m, P, U(p), D(a), D(R), D(r), D(W), D(beta), D(delta), D(G))
    # draws of a valid posterior, evolved with G
    m2, C2, n2, s2 = random_state(rng, m, P, p, off_block=False)
    for j in range(m):
        m2[p[j]:, j] = 0.0
    lam_o, th_o, capped = oracle.sample(p, m2, C2, n2, s2, n, seed, epoch)
    assert capped == 0
    th_dm = np.ascontiguousarray(th_o.transpose(1, 2, 0))
    W2 = np.zeros((P, P, m), order="F")
    for j in range(m):
        A = rng.normal(0, 0.05, (p[j], p[j]))
        W2[: p[j], : p[j], j] = A @ A.T + 1e-4 * np.eye(p[j])
    c_t = f64(rng.uniform(0.002, 0.02, m))
    r_t = f64(rng.uniform(8, 20, m))
    beta2 = f64(np.full(m, 0.95)); beta2[0] = 1.0
    ev_epoch = epoch + 1
    lam_ev, _, capped = oracle.evolve(p, W2, r_t, c_t, beta2, lam_o, th_o, seed, ev_epoch, compat=3,
                                      G=G)
    om = philox_normals(seed, ev_epoch, TAG_OMEGA, n, m, P)
    th_ev_ref = th_dm.copy()
    L.ref_evolve_theta_g(m, P, U(p), D(W2), D(c_t), n, D(np.ascontiguousarray(lam_ev)),
                         D(np.ascontiguousarray(om)), D(G), D(th_ev_ref))
    np.savez(OUT / f"{name}_evo.npz", p=p, sp=sp, m_t=m_t, C_t=C_t, n_t=n_t, beta=beta, delta=delta,
             G=G, evo_a=a, evo_R=R, evo_r=r, evo_W=W, m2=m2, C2=C2, n2=n2, s2=s2, n=n, seed=seed,
             epoch=epoch, W2=W2, c_t=c_t, r_t=r_t, beta2=beta2, ev_epoch=ev_epoch,
             lambdas_ev=np.ascontiguousarray(lam_ev), thetas_ev_ref=th_ev_ref)


def case_samplers(L, rng):
    """make_gamma2 and make_beta on supplied uniforms/normals (n_loops = 2)."""
    m, n, loops = 3, 1000, 2
    n_t = f64([2.0, 6.0, 40.0]); s_t = f64([0.5, 0.01, 2.0])
    uni = rng.uniform(0, 1, loops * n * m); nor = rng.normal(0, 1, loops * n * m)
    g = np.zeros((n, m))
    L.ref_make_gamma2(m, n, loops, D(uni), D(nor), D(n_t), D(s_t), D(g))
    ga = rng.gamma(5.0, 1.0, (n, m))
    r_t = f64([18.0, 3.0, 30.0]); beta = f64([0.95, 0.8, 1.0])
    uni2 = rng.uniform(0, 1, loops * n * m); nor2 = rng.normal(0, 1, loops * n * m)
    b = ga.copy()
    L.ref_make_beta(m, n, loops, D(uni2), D(nor2), D(r_t), D(beta), D(b))
    np.savez(OUT / "samplers.npz", n_t=n_t, s_t=s_t, uniforms=uni, normals=nor, gammas=g,
             ga=ga, r_t=r_t, beta=beta, uniforms2=uni2, normals2=nor2, betas=b, loops=loops)


def case_psi(L):
    xs = np.array([0.3, 0.5, 0.9, 1.0, 1.5, 2.0, 3.7, 5.0, 10.0, 25.0, 100.0, 1e3])
    np.savez(OUT / "psi.npz", x=xs, psi=np.array([L.ref_psi(v) for v in xs]),
             psi1=np.array([L.ref_psi1(v) for v in xs]))


def main():
    L = ref_lib()
    rng = np.random.default_rng(20261203)
    p, sp = readme_parents()
    case_posterior_prior(L, rng, "readme", p, sp)
    p2, sp2 = random_parents(rng, 20, 3, 5)
    case_posterior_prior(L, rng, "m20", p2, sp2)
    case_sampling_vb_forecast(L, rng, "readme", p, sp, n=400, seed=1234, epoch=7)
    case_sampling_vb_forecast(L, rng, "m20", p2, sp2, n=300, seed=0xDEADBEEF12345, epoch=3)
    case_samplers(L, rng)
    case_psi(L)
    case_evolution_matrix(L, rng, "m20", p2, sp2, n=200, seed=77, epoch=5)
    for f in sorted(OUT.glob("*.npz")):
        print(f.name, f.stat().st_size)


if __name__ == "__main__":
    main()
