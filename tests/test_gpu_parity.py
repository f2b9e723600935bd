"""Parity of the GB300 CUDA path with the oracle and the reference-kernel fixtures.

Every call goes through the C ABI (ctypes -> libsgdlm_gb300.so).  Tolerances:
  FP64 mode  : deterministic steps 1e-12 relative; sampled steps compared draw by
               draw on identical Philox streams, 1e-9 relative (CUDA's and glibc's
               log/sin/cos differ in the last bits, which the LU and moments carry).
  mixed mode : draws are FP32 (normals within ~1e-6 relative of FP64); per-draw
               log|det| within 2e-4 absolute of the FP64 oracle on the same draws;
               VB moments within 1e-3 relative; refined forecast solves within 1e-5
               relative of the FP64 solve of the same draws.
"""
import ctypes

import numpy as np
import pytest

import oracle
from gpusgdlm_gb300 import SGDLM
from oracle_model import OracleSGDLM

pytestmark = pytest.mark.gpu
NAMES = ["readme", "m20"]


def na_sp(sp, m):
    s = sp.astype(np.float64)
    s[sp >= m * m] = np.nan
    return s


def model_from(g, precision, seed=1234, epoch=0, beta=None, delta=None):
    P, m = g["sp"].shape
    s = SGDLM(1, strict=True, precision=precision)
    s.setSimultaneousParents(g["p"], na_sp(g["sp"], m))
    b = np.full(m, 0.95) if beta is None else beta
    d = np.full((P, P, m), 0.97) if delta is None else delta
    s.setDiscountFactors(b, d)
    s.setRngState(seed, epoch)
    return s


@pytest.mark.parametrize("name", NAMES)
def test_posterior_prior_match_reference(built_lib, golden, name):
    g = golden(f"{name}_posterior_prior.npz")
    s = model_from(g, "fp64", beta=g["beta"], delta=g["delta"])
    s.setPriorParameters(g["m_t"], g["C_t"], g["n_t"], g["s_t"])
    s.computePosterior(g["y"], g["F"])
    post = s.getParameters()
    np.testing.assert_allclose(post["m"], g["post_m"], rtol=1e-12, atol=1e-15)
    np.testing.assert_allclose(post["C"], g["post_C"], rtol=1e-12, atol=1e-15)
    np.testing.assert_array_equal(post["n"], g["post_n"])
    np.testing.assert_allclose(post["s"], g["post_s"], rtol=1e-12)
    s.computePrior()
    pr = s.getParameters()
    np.testing.assert_allclose(pr["C"], g["prior_C"], rtol=1e-12, atol=1e-15)
    np.testing.assert_array_equal(pr["n"], g["prior_n"])


@pytest.mark.parametrize("name", NAMES)
def test_vb_fp64_matches_reference(built_lib, golden, name):
    g = golden(f"{name}_vb_forecast.npz")
    n, seed, epoch = int(g["n"]), int(g["seed"]), int(g["epoch"])
    s = model_from(g, "fp64", seed=seed, epoch=epoch)
    s.setPosteriorParameters(g["m_t"], g["C_t"], g["n_t"], g["s_t"])
    vb = s.computeVBPosterior(n, n)
    d = s.getDraws()
    lam_o, th_o, _ = oracle.sample(g["p"], g["m_t"], g["C_t"], g["n_t"], g["s_t"], n, seed, epoch)
    np.testing.assert_allclose(d["lambdas"], lam_o.T, rtol=1e-13)
    np.testing.assert_allclose(d["thetas"], th_o.transpose(0, 2, 1), rtol=1e-12, atol=1e-14)
    np.testing.assert_allclose(vb["IS_weights"], g["w"], rtol=1e-9)
    np.testing.assert_allclose(vb["sum_det_weights"], g["sum_w"], rtol=1e-9)
    np.testing.assert_allclose(vb["m"], g["vb_m"], rtol=1e-9, atol=1e-13)
    np.testing.assert_allclose(vb["C"], g["vb_C"], rtol=1e-9, atol=1e-15)
    np.testing.assert_allclose(vb["n"], g["vb_n"], rtol=1e-9)
    np.testing.assert_allclose(vb["s"], g["vb_s"], rtol=1e-9)


@pytest.mark.parametrize("name", NAMES)
def test_vb_mixed_matches_oracle_on_device_draws(built_lib, golden, name):
    g = golden(f"{name}_vb_forecast.npz")
    n, seed, epoch = int(g["n"]), int(g["seed"]), int(g["epoch"])
    s = model_from(g, "mixed", seed=seed, epoch=epoch)
    s.setPosteriorParameters(g["m_t"], g["C_t"], g["n_t"], g["s_t"])
    vb = s.computeVBPosterior(n, n)
    d = s.getDraws()
    lam_o, th_o, _ = oracle.sample(g["p"], g["m_t"], g["C_t"], g["n_t"], g["s_t"], n, seed, epoch)
    # FP32 draws of the same stream
    np.testing.assert_allclose(d["lambdas"], lam_o.T, rtol=2e-5)
    np.testing.assert_allclose(d["thetas"], th_o.transpose(0, 2, 1), rtol=2e-4, atol=2e-5)
    lam = np.asfortranarray(d["lambdas"].T)
    th = np.asfortranarray(d["thetas"].transpose(0, 2, 1))
    ld = oracle.logdet(g["sp"], th)
    np.testing.assert_allclose(d["log_dets"], ld, rtol=0, atol=2e-4)
    w, sw = oracle.weights(ld)
    np.testing.assert_allclose(vb["IS_weights"], w, rtol=5e-4)
    ref = oracle.vb(g["p"], g["n_t"], g["s_t"], w, lam, th)
    np.testing.assert_allclose(vb["m"], ref["m"], rtol=1e-3, atol=1e-5)
    np.testing.assert_allclose(vb["C"], ref["C"], rtol=1e-3, atol=1e-7)
    np.testing.assert_allclose(vb["n"], ref["n"], rtol=1e-3)
    np.testing.assert_allclose(vb["s"], ref["s"], rtol=1e-3)


@pytest.mark.parametrize("name", NAMES)
def test_forecast_fp64_matches_reference(built_lib, golden, name):
    g = golden(f"{name}_vb_forecast.npz")
    n, seed, epoch = int(g["n"]), int(g["seed"]), int(g["epoch"])
    s = model_from(g, "fp64", seed=seed, epoch=epoch)
    s.setPriorParameters(g["m_t"], g["C_t"], g["n_t"], g["s_t"])
    out = s.computeForecastDebug(n, n, g["x"])
    np.testing.assert_allclose(out["y"], g["y_ref"].T, rtol=1e-9, atol=1e-11)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_forecast_into_page_locked_buffer(built_lib, golden, precision):
    """A page-locked destination receives the forecast draws straight from the LU
    kernels; they equal the copied-back draws of a pageable destination."""
    torch = pytest.importorskip("torch")
    import ctypes as C

    g = golden("readme_vb_forecast.npz")
    n, seed, epoch = int(g["n"]), int(g["seed"]), int(g["epoch"])
    P, m = g["sp"].shape
    s = model_from(g, precision, seed=seed, epoch=epoch)
    s.setPriorParameters(g["m_t"], g["C_t"], g["n_t"], g["s_t"])
    assert s._ensure_sim(n, n)
    lib, h = s._lib, s._h
    dp = C.POINTER(C.c_double)
    x = np.asfortranarray(g["x"], dtype=np.float64)

    def run(buf):
        s.setRngState(seed, epoch)
        assert lib.sgdlm_init_forecast_priors(h) == 0
        assert lib.sgdlm_compute_forecast(h, buf.ctypes.data_as(dp), x.ctypes.data_as(dp),
                                          None, None, 0) == 0

    pageable = np.full(m * n, np.nan)
    run(pageable)
    locked = torch.full((m * n,), float("nan"), dtype=torch.float64).pin_memory().numpy()
    run(locked)
    assert np.isfinite(pageable).all()
    np.testing.assert_array_equal(locked, pageable)


@pytest.mark.parametrize("name", NAMES)
def test_forecast_mixed_refined(built_lib, golden, name):
    g = golden(f"{name}_vb_forecast.npz")
    n, seed, epoch = int(g["n"]), int(g["seed"]), int(g["epoch"])
    s = model_from(g, "mixed", seed=seed, epoch=epoch)
    s.setPriorParameters(g["m_t"], g["C_t"], g["n_t"], g["s_t"])
    out = s.computeForecastDebug(n, n, g["x"])
    lam = np.asfortranarray(out["lambdas"].T)
    th = np.asfortranarray(out["thetas"].transpose(0, 2, 1))
    y, _ = oracle.forecast(g["sp"], lam, th, g["x"], seed, epoch)
    np.testing.assert_allclose(out["y"], y, rtol=1e-5, atol=1e-6)


@pytest.mark.parametrize("compat", [3, 0])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_multistep_forecast_matches_oracle(built_lib, golden, precision, compat):
    """K = 3 step forecasts (evolution between steps).  compat = 3 reproduces the
    reference's Beta sampler, which returns NaN for shapes below 1/3; a dense solve
    spreads such a NaN over the whole draw, the sparse elimination only over the
    entries it reaches, so there only finite entries are compared."""
    g = golden("m20_vb_forecast.npz")
    P, m = g["sp"].shape
    n, seed, epoch = 256, 99, 5
    x3 = np.asfortranarray(np.stack([g["x"] * (1 + 0.1 * k) for k in range(3)], axis=2))
    s = model_from(g, precision, seed=seed, epoch=epoch)
    s.setCompat(compat)
    s.setPosteriorParameters(g["m_t"], g["C_t"], g["n_t"], g["s_t"])
    s.computePrior()
    y = s.computeForecast(n, n, x3)
    o = OracleSGDLM(g["p"], g["sp"], np.full(m, 0.95), np.full((P, P, m), 0.97), seed=seed,
                    epoch=epoch, compat=compat)
    o.set_parameters(g["m_t"], g["C_t"], g["n_t"], g["s_t"])
    o.prior()
    yo = o.forecast(n, x3)
    assert y.shape == (m, n, 3)
    rtol, atol = (1e-8, 1e-10) if precision == "fp64" else (2e-3, 2e-4)
    if compat == 0:
        assert np.isfinite(y).all() and np.isfinite(yo).all()
        np.testing.assert_allclose(y, yo, rtol=rtol, atol=atol)
    else:
        both = np.isfinite(y) & np.isfinite(yo)
        assert both[:, :, 0].all()  # the first step has no evolution
        np.testing.assert_allclose(y[both], yo[both], rtol=rtol, atol=atol)
        assert np.all(np.isfinite(y)[np.isfinite(yo)])  # finite in the oracle -> finite here
    assert s.getRngState()[1] == epoch + 5


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_multistep_forecast_block_lu_matches_oracle(built_lib, precision):
    """K = 3 step forecasts at m = 96, above the warp-per-draw LU's m <= 32: the
    draws' Gamma entries reach the block LU and the iterative solve through the
    sampler's and the evolution's draw-major Gamma copy.  Corrected samplers
    (compat 0), an informative posterior (so most draws take the fast path and
    the iterative solve), against the oracle on the same streams."""
    import bench

    wl = bench.make_workload(m=96, kmax=10, T=4, seed=777)
    m, P = wl["m"], wl["P"]
    rng = np.random.default_rng(5)
    mt = np.asfortranarray(rng.normal(0.0, 0.05, (P, m)))
    Ct = np.asfortranarray(np.repeat((1e-3 * np.eye(P))[:, :, None], m, axis=2))
    nt, st = np.full(m, 50.0), np.full(m, 0.0025)
    n, seed, epoch = 256, 31, 2
    x3 = np.asfortranarray(np.stack([wl["F_of"](1 + k, False) for k in range(3)], axis=2))
    s = SGDLM(1, strict=True, precision=precision)
    s.setCompat(0)
    s.setSimultaneousParents(wl["p"], na_sp(wl["sp"], m))
    s.setDiscountFactors(np.full(m, 0.97), np.full((P, P, m), 0.98))
    s.setRngState(seed, epoch)
    s.setPosteriorParameters(mt, Ct, nt, st)
    s.computePrior()
    y = s.computeForecast(n, n, x3)
    s.close()
    o = OracleSGDLM(wl["p"], wl["sp"], np.full(m, 0.97), np.full((P, P, m), 0.98), seed=seed,
                    epoch=epoch, compat=0)
    o.set_parameters(mt, Ct, nt, st)
    o.prior()
    yo = o.forecast(n, x3)
    assert y.shape == (m, n, 3)
    assert np.isfinite(y).all() and np.isfinite(yo).all()
    rtol, atol = (1e-8, 1e-10) if precision == "fp64" else (2e-3, 2e-4)
    np.testing.assert_allclose(y, yo, rtol=rtol, atol=atol)


def test_evo_prior_matches_reference(built_lib, golden):
    """computeEvoPrior against the reference's kernels (fixture m20_evo): a = G m and
    R = G R G' with the reference's cut-offs, FP64."""
    g = golden("m20_evo.npz")
    P, m = g["sp"].shape
    s = model_from(g, "fp64", beta=g["beta"], delta=g["delta"])
    s.setPosteriorParameters(g["m_t"], g["C_t"], g["n_t"], np.ones(m))
    s.computeEvoPrior(g["G"])
    assert s.isPrior()
    prm = s.getParameters()
    np.testing.assert_array_equal(prm["n"], g["evo_r"])
    np.testing.assert_allclose(prm["m"], g["evo_a"], rtol=1e-12, atol=1e-15)
    np.testing.assert_allclose(prm["C"], g["evo_R"], rtol=1e-12, atol=1e-15)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_evo_forecast_matches_oracle(built_lib, golden, precision):
    """computeEvoForecast, K = 3 steps with one evolution matrix per step: the draws
    evolve as theta = G theta + chol(W)' omega between steps."""
    g = golden("m20_vb_forecast.npz")
    ge = golden("m20_evo.npz")
    P, m = g["sp"].shape
    n, seed, epoch = 256, 41, 2
    x3 = np.asfortranarray(np.stack([g["x"] * (1 + 0.1 * k) for k in range(3)], axis=2))
    G4 = np.asfortranarray(np.stack([ge["G"] * (1 - 0.05 * k) for k in range(3)], axis=3))
    s = model_from(g, precision, seed=seed, epoch=epoch)
    s.setCompat(0)
    s.setPosteriorParameters(g["m_t"], g["C_t"], g["n_t"], g["s_t"])
    s.computePrior()
    y = s.computeEvoForecast(n, n, x3, G4)
    o = OracleSGDLM(g["p"], g["sp"], np.full(m, 0.95), np.full((P, P, m), 0.97), seed=seed,
                    epoch=epoch, compat=0)
    o.set_parameters(g["m_t"], g["C_t"], g["n_t"], g["s_t"])
    o.prior()
    yo = o.forecast(n, x3, G4)
    assert y.shape == (m, n, 3)
    assert np.isfinite(y).all() and np.isfinite(yo).all()
    rtol, atol = (1e-8, 1e-10) if precision == "fp64" else (2e-3, 2e-4)
    np.testing.assert_allclose(y, yo, rtol=rtol, atol=atol)
    # the evolution matrix matters: without it the later steps differ
    assert not np.allclose(y[:, :, 2], s.computeForecast(n, n, x3)[:, :, 2], rtol=1e-3)


def readme_inputs(T, seed=20261203):
    """The README scenario (README.md:48-154) as arrays."""
    m = 6
    counts = [2, 0, 1, 3, 1, 2]
    sim = [[6], [1, 6, 4], [], [1, 2], [], [2, 4]]
    p = np.array([c + len(s) for c, s in zip(counts, sim)])
    P = int(p.max())
    sp = np.full((P, m), np.nan)
    for j in range(m):
        for t, par in enumerate(sim[j]):
            sp[counts[j] + t, j] = j + m * (par - 1)
    rng = np.random.default_rng(seed)
    true_means = np.repeat([0, 0.1, 0.2, 0.15, 0.05], T // 5)
    y = rng.normal(true_means[:, None], 0.025, size=(T, m))

    def predictors(t, yrow):
        F = np.zeros((P, m), order="F")
        F[0:2, 0] = [1, y[t - 1, 0]]
        F[0, 2] = 1
        F[0:3, 3] = [1, y[t - 1, 3], true_means[t]]
        F[0, 4] = 1
        F[0:2, 5] = [1, y[t - 1, 0]]
        if yrow is not None:
            for j in range(m):
                for t2, par in enumerate(sim[j]):
                    F[counts[j] + t2, j] = yrow[par - 1]
        return F

    beta = np.full(m, 0.95)
    Delta = np.full((P, P, m), 0.95)
    Delta[:, :, 2] = 0.7
    Delta[:, :, 4] = 0.9999
    return dict(m=m, P=P, p=p, sp=sp, y=y, predictors=predictors, beta=beta, Delta=Delta)


def test_readme_scenario_fp64_matches_oracle(built_lib):
    """20 steps of the README loop, GPU vs oracle on identical streams."""
    T, n = 20, 2000
    d = readme_inputs(100)
    m, P = d["m"], d["P"]
    s = SGDLM(1, strict=True, precision="fp64")
    s.setSimultaneousParents(d["p"], d["sp"])
    s.setDiscountFactors(d["beta"], d["Delta"])
    a, R = np.zeros((P, m)), np.repeat((0.05 * np.eye(P))[:, :, None], m, axis=2)
    s.setPriorParameters(a, R, np.full(m, 3.0), np.full(m, 0.01))
    s.setRngState(777, 0)
    spu = np.where(np.isnan(d["sp"]), 2147483648, np.nan_to_num(d["sp"])).astype(np.uint32)
    o = OracleSGDLM(d["p"], spu, d["beta"], d["Delta"], seed=777, epoch=0)
    o.set_parameters(a, R, np.full(m, 3.0), np.full(m, 0.01))
    for t in range(1, T):
        F = d["predictors"](t, d["y"][t])
        s.computePosterior(d["y"][t], F)
        o.posterior(d["y"][t], F)
        vb = s.computeVBPosterior(n, n)
        vo = o.vb(n)
        np.testing.assert_allclose(vb["IS_weights"], vo["IS_weights"], rtol=1e-8)
        ess = 1 / np.sum(vb["IS_weights"] ** 2)
        if ess > n / 2:  # README.md:131
            s.setPosteriorParameters(vb["m"], vb["C"], vb["n"], vb["s"])
            o.set_parameters(vo["m"], vo["C"], vo["n"], vo["s"])
        s.computePrior()
        o.prior()
        Fn = d["predictors"](t + 1, None)
        yf = s.computeForecast(n, n, Fn)
        yo = o.forecast(n, Fn)
        np.testing.assert_allclose(yf, yo, rtol=1e-7, atol=1e-9)
    gp = s.getParameters()
    np.testing.assert_allclose(gp["m"], o.m_t, rtol=1e-7, atol=1e-10)
    np.testing.assert_allclose(gp["C"], o.C_t, rtol=1e-7, atol=1e-12)
    np.testing.assert_allclose(gp["n"], o.n_t, rtol=1e-9)
    np.testing.assert_allclose(gp["s"], o.s_t, rtol=1e-7)


def test_state_machine_and_errors(built_lib, golden):
    g = golden("readme_vb_forecast.npz")
    P, m = g["sp"].shape
    s = SGDLM(1, strict=False, precision="mixed")
    # as in RcppWrapper.cpp:302-306 the dimension check (m = 0 so far) comes first
    s.computePosterior(np.zeros(m), np.zeros((P, m)))
    assert s.last_status == 1
    # the engine itself refuses before initMemory (HostWrapperImpl.cu:1240-1246)
    y, F = np.zeros(m), np.zeros((P, m), order="F")
    dp = ctypes.POINTER(ctypes.c_double)
    st = s._lib.sgdlm_compute_posterior(s._h, y.ctypes.data_as(dp), F.ctypes.data_as(dp))
    assert st == 2  # NOT_INIT
    s.setSimultaneousParents(g["p"], na_sp(g["sp"], m))
    assert s.last_status == 0
    s.setDiscountFactors(np.full(m, 0.9), np.full((P, P, m + 1), 0.9))
    assert s.last_status == 1  # BAD_DIM
    s.setPosteriorParameters(g["m_t"], g["C_t"], g["n_t"], g["s_t"])
    s.computePosterior(np.zeros(m), np.zeros((P, m)))
    assert s.last_status == 3  # WRONG_STATE: posterior on posterior
    before = s.getParameters()
    s.computeForecast(100, 100, g["x"])
    assert s.last_status == 3  # forecast needs the prior
    after = s.getParameters()
    np.testing.assert_array_equal(before["C"], after["C"])
    s.computePrior()
    assert s.isPrior()
    assert s.computeVBPosterior(100, 100) is None and s.last_status == 3
    bad = na_sp(g["sp"], m)
    bad[0, 0] = 0.0  # diagonal entry of (I - Gamma)
    s.setSimultaneousParents(g["p"], bad)
    assert s.last_status == 6
    # round trips
    par = s.getSimultaneousParents()
    np.testing.assert_array_equal(par["p"], g["p"])
    np.testing.assert_array_equal(np.isnan(par["sp"]), g["sp"] >= m * m)
    df = s.getDiscountFactors()
    np.testing.assert_array_equal(df["beta"], np.zeros(m))  # the bad call changed nothing
    s.setLogLevel(7)
    assert s.getLogLevel() == 5
    s.clearSimulationMemory()
    assert s.nsim == 0


def test_rng_checkpoint_reproducible(built_lib, golden):
    g = golden("m20_vb_forecast.npz")
    outs = []
    for _ in range(2):
        s = model_from(g, "mixed", seed=42, epoch=11)
        s.setPosteriorParameters(g["m_t"], g["C_t"], g["n_t"], g["s_t"])
        outs.append(s.computeVBPosterior(500, 500))
        assert s.getRngState() == (42, 12)
    for k in ("m", "C", "n", "s", "IS_weights"):
        np.testing.assert_array_equal(outs[0][k], outs[1][k])


@pytest.mark.parametrize("n", [1, 37, 1000])
def test_ragged_draw_counts(built_lib, golden, n):
    g = golden("readme_vb_forecast.npz")
    s = model_from(g, "fp64", seed=5, epoch=0)
    s.setPosteriorParameters(g["m_t"], g["C_t"], g["n_t"], g["s_t"])
    vb = s.computeVBPosterior(n, n)
    lam, th, _ = oracle.sample(g["p"], g["m_t"], g["C_t"], g["n_t"], g["s_t"], n, 5, 0)
    ld = oracle.logdet(g["sp"], th)
    w, sw = oracle.weights(ld)
    np.testing.assert_allclose(vb["IS_weights"], w, rtol=1e-9)
    np.testing.assert_allclose(vb["sum_det_weights"], sw, rtol=1e-9)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_draw_buffers_kept_across_smaller_counts(built_lib, precision):
    """The per-draw buffers only grow: a call with fewer draws after one with more
    reuses the larger allocations (their old contents included) and must give
    bit for bit what a freshly allocated engine gives (m = 96: block LU, iterative
    forecast solve, the draw-major Gamma copy)."""
    import bench

    wl = bench.make_workload(m=96, kmax=10, T=4, seed=778)
    m, P = wl["m"], wl["P"]
    rng = np.random.default_rng(6)
    mt = np.asfortranarray(rng.normal(0.0, 0.05, (P, m)))
    Ct = np.asfortranarray(np.repeat((1e-3 * np.eye(P))[:, :, None], m, axis=2))
    nt, st = np.full(m, 50.0), np.full(m, 0.0025)
    x = wl["F_of"](2, False)

    def run(first):
        s = SGDLM(1, strict=True, precision=precision)
        s.setSimultaneousParents(wl["p"], na_sp(wl["sp"], m))
        s.setDiscountFactors(np.full(m, 0.97), np.full((P, P, m), 0.98))
        if first:
            s.setRngState(99, 0)
            s.setPosteriorParameters(mt, Ct, nt, st)
            s.computeVBPosterior(first, first)   # allocates for `first` draws
            s.computePrior()
            s.computeForecast(first, first, x)
        s.setRngState(31, 3)
        s.setPosteriorParameters(mt, Ct, nt, st)
        vb = s.computeVBPosterior(700, 700)
        s.computePrior()
        y = s.computeForecast(300, 300, x)
        s.close()
        return vb, y

    vb0, y0 = run(0)
    vb1, y1 = run(5000)
    for k in ("m", "C", "n", "s", "IS_weights"):
        np.testing.assert_array_equal(vb1[k], vb0[k])
    np.testing.assert_array_equal(y1, y0)


def test_single_series_and_empty_predictors(built_lib):
    """m = 1 with no parents, and a series with p_j = 0."""
    s = SGDLM(1, strict=True, precision="fp64")
    s.setSimultaneousParents([2, 0], np.full((2, 2), np.nan))
    s.setDiscountFactors([0.95, 0.95], np.full((2, 2, 2), 0.95))
    C = np.zeros((2, 2, 2)); C[:, :, 0] = 0.1 * np.eye(2)
    s.setPosteriorParameters(np.array([[0.1, 0.0], [0.2, 0.0]]), C, [10.0, 10.0], [0.01, 0.02])
    s.setRngState(3, 0)
    vb = s.computeVBPosterior(300, 300)
    # no simultaneous parents: det = 1 for every draw, uniform weights
    np.testing.assert_allclose(vb["IS_weights"], 1.0 / 300, rtol=1e-14)
    np.testing.assert_allclose(vb["sum_det_weights"], 300.0, rtol=1e-14)
    assert np.all(vb["C"][:, :, 1] == 0.0)
    o = OracleSGDLM([2, 0], np.full((2, 2), 2147483648, dtype=np.uint32), [0.95, 0.95],
                    np.full((2, 2, 2), 0.95), seed=3, epoch=0)
    o.set_parameters(np.array([[0.1, 0.0], [0.2, 0.0]]), C, [10.0, 10.0], [0.01, 0.02])
    vo = o.vb(300)
    np.testing.assert_allclose(vb["n"], vo["n"], rtol=1e-9)
    np.testing.assert_allclose(vb["s"], vo["s"], rtol=1e-9)


@pytest.mark.parametrize("levels", [0, 4])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_pivoting_fallback(built_lib, precision, levels):
    """A large coefficient below the diagonal: the dense no-pivot pass (levels = 0)
    must hand every draw to the partial-pivoting redo; the sparse elimination
    (levels = 4) eliminates node 1 first, where the multiplier is small."""
    m, P = 3, 1
    sp = np.array([[0 + 3 * 1, 1 + 3 * 0, 2 + 3 * 0]], dtype=np.float64)  # 0<-1, 1<-0, 2<-0
    s = SGDLM(1, strict=True, precision=precision)
    s.setWarpLu(False)  # the block LU kernels (m <= 32 takes the warp path by default)
    s.setSimultaneousParents([1, 1, 1], sp)
    s.setEliminationLevels(levels)
    s.setDiscountFactors(np.full(m, 0.95), np.full((P, P, m), 0.95))
    mt = np.array([[0.3, 20.0, -15.0]])
    C = np.full((1, 1, m), 1e-4)
    s.setPosteriorParameters(mt, C, np.full(m, 20.0), np.full(m, 1.0))
    s.setRngState(8, 0)
    vb = s.computeVBPosterior(200, 200)
    st = s.getStats()
    assert st["draws_pivoted"] == (200 if levels == 0 else 0)
    d = s.getDraws()
    th = np.asfortranarray(d["thetas"].transpose(0, 2, 1))
    spu = sp.astype(np.uint32)
    ld = oracle.logdet(spu, th)
    np.testing.assert_allclose(d["log_dets"], ld, rtol=1e-5 if precision == "mixed" else 1e-12,
                               atol=1e-5 if precision == "mixed" else 1e-13)
    assert np.isfinite(vb["n"]).all()


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_pivoting_fallback_forecast(built_lib, precision):
    """Forecast draws through the partial-pivoting redo (levels = 0 and a
    multiplier of 20 below the diagonal): the permuted solve plus one FP64
    refinement gives y = (I - Gamma)^-1 nu of the oracle."""
    m, P = 3, 1
    sp = np.array([[0 + 3 * 1, 1 + 3 * 0, 2 + 3 * 0]], dtype=np.float64)
    s = SGDLM(1, strict=True, precision=precision)
    s.setWarpLu(False)  # the block LU kernels (m <= 32 takes the warp path by default)
    s.setSimultaneousParents([1, 1, 1], sp)
    s.setEliminationLevels(0)
    s.setDiscountFactors(np.full(m, 0.95), np.full((P, P, m), 0.95))
    s.setPriorParameters(np.array([[0.3, 20.0, -15.0]]), np.full((1, 1, m), 1e-4),
                         np.full(m, 20.0), np.full(m, 1.0))
    s.setRngState(8, 0)
    x = np.zeros((P, m), order="F")
    out = s.computeForecastDebug(256, 256, x)
    assert s.getStats()["draws_pivoted"] == 256
    lam = np.asfortranarray(out["lambdas"].T)
    th = np.asfortranarray(out["thetas"].transpose(0, 2, 1))
    y, _ = oracle.forecast(sp.astype(np.uint32), lam, th, x, 8, 0)
    # y_1 = nu_1 + 20 y_0 cancels terms of size ~6 down to ~1e-2: FP32 factors plus
    # one FP64-residual refinement leave absolute errors of a few 1e-6 there
    tol = dict(rtol=1e-5, atol=1e-5) if precision == "mixed" else dict(rtol=1e-10, atol=1e-12)
    np.testing.assert_allclose(out["y"], y, **tol)


@pytest.mark.parametrize("g01,full", [(100.0, False), (1.0e5, True)])
@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_pivoting_redo_core_and_full(built_lib, precision, g01, full):
    """The redo keeps the sparse levels and pivots in the dense core, unless a
    level multiplier is huge.  Parents 0<-1, 1<-0, 2<-0: level 0 eliminates nodes
    1 and 2 (pivots 1), the core is node 0 and the level multiplier is
    -Gamma_01.  Gamma_01 = 100 fails the fast pass's check (8) and is redone in
    the core; Gamma_01 = 1e5 exceeds the levels' bound (65536) and is pivoted over
    the full matrix.  log|det| and the forecasts against the oracle."""
    m, P = 3, 1
    sp = np.array([[0 + 3 * 1, 1 + 3 * 0, 2 + 3 * 0]], dtype=np.float64)
    s = SGDLM(1, strict=True, precision=precision)
    s.setWarpLu(False)  # the block LU kernels (m <= 32 takes the warp path by default)
    s.setSimultaneousParents([1, 1, 1], sp)
    s.setEliminationLevels(4)
    s.setDiscountFactors(np.full(m, 0.95), np.full((P, P, m), 0.95))
    mt = np.array([[g01, 20.0, -15.0]])
    C = np.full((1, 1, m), 1e-6)
    s.setPosteriorParameters(mt, C, np.full(m, 20.0), np.full(m, 1.0))
    s.setRngState(9, 0)
    s.computeVBPosterior(200, 200)
    assert s.getEliminationInfo()["levels"] == 1
    st = s.getStats()
    assert st["draws_pivoted"] == 200
    assert st["draws_pivoted_full"] == (200 if full else 0)
    d = s.getDraws()
    th = np.asfortranarray(d["thetas"].transpose(0, 2, 1))
    spu = sp.astype(np.uint32)
    tol = dict(rtol=1e-5, atol=1e-5) if precision == "mixed" else dict(rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(d["log_dets"], oracle.logdet(spu, th), **tol)
    # forecasts of the same kind of draws (the iterative solve diverges on them)
    s.setPriorParameters(mt, C, np.full(m, 20.0), np.full(m, 1.0))
    s.setRngState(10, 0)
    x = np.zeros((P, m), order="F")
    out = s.computeForecastDebug(256, 256, x)
    st = s.getStats()
    assert st["draws_pivoted"] == 256
    assert st["draws_pivoted_full"] == (256 if full else 0)
    lam = np.asfortranarray(out["lambdas"].T)
    th = np.asfortranarray(out["thetas"].transpose(0, 2, 1))
    y, _ = oracle.forecast(spu, lam, th, x, 10, 0)
    # normwise per draw: |y| reaches ~1e4 / 20 on the components that the large
    # coefficient couples
    err = np.abs(out["y"] - y).max(axis=0) / np.abs(y).max(axis=0)
    assert err.max() <= (1e-5 if precision == "mixed" else 1e-11)
    s.close()


def test_fused_device_step_matches_api_sequence(built_lib):
    torch = pytest.importorskip("torch")
    d = readme_inputs(100)
    m, P, n = d["m"], d["P"], 1024
    a, R = np.zeros((P, m)), np.repeat((0.05 * np.eye(P))[:, :, None], m, axis=2)

    def fresh():
        s = SGDLM(1, strict=True, precision="mixed")
        s.setSimultaneousParents(d["p"], d["sp"])
        s.setDiscountFactors(d["beta"], d["Delta"])
        s.setPriorParameters(a, R, np.full(m, 3.0), np.full(m, 0.01))
        s.setRngState(55, 0)
        return s

    s1, s2 = fresh(), fresh()
    s2._ensure_sim(n, n)
    dev = torch.device("cuda:0")
    for t in range(1, 6):
        F = d["predictors"](t, d["y"][t])
        Fn = d["predictors"](t + 1, None)
        # API sequence, ESS gate as in README.md:131 with threshold n/2
        s1.computePosterior(d["y"][t], F)
        vb = s1.computeVBPosterior(n, n)
        if 1 / np.sum(vb["IS_weights"] ** 2) > n / 2:
            s1.setPosteriorParameters(vb["m"], vb["C"], vb["n"], vb["s"])
        s1.computePrior()
        y1 = s1.computeForecast(n, n, Fn)
        # fused device step
        ty = torch.tensor(d["y"][t], dtype=torch.float64, device=dev)
        tF = torch.tensor(np.asfortranarray(F).ravel(order="F"), dtype=torch.float64, device=dev)
        tx = torch.tensor(np.asfortranarray(Fn).ravel(order="F"), dtype=torch.float64, device=dev)
        tyout = torch.zeros(n * m, dtype=torch.float64, device=dev)
        tst = torch.zeros(8, dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        assert s2.filterStepDevice(ty.data_ptr(), tF.data_ptr(), tx.data_ptr(), n / 2,
                                   tyout.data_ptr(), None, tst.data_ptr())
        s2.synchronize()
        y2 = tyout.cpu().numpy().reshape(m, n, order="F")
        np.testing.assert_array_equal(y1, y2)
    p1, p2 = s1.getParameters(), s2.getParameters()
    for k in ("m", "C", "n", "s"):
        np.testing.assert_array_equal(p1[k], p2[k])


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_benchmark_size_m400(built_lib, precision):
    """m = 400, p_j <= 20 (the benchmark's shape): a subset of draws against the oracle,
    plus size-independent properties over all draws."""
    import bench

    wl = bench.make_workload(m=400, T=4, seed=11)
    m, P, n = wl["m"], wl["P"], 1024
    s = SGDLM(1, strict=True, precision=precision)
    s.setSimultaneousParents(wl["p"], np.where(wl["sp"] >= m * m, np.nan, wl["sp"]).astype(float))
    s.setDiscountFactors(np.full(m, 0.97), np.full((P, P, m), 0.98))
    a, R, r, c = bench.prior_arrays(m, P)
    s.setPriorParameters(a, R, r, c)
    s.setRngState(21, 0)
    s.computePosterior(wl["y"][1], wl["F_of"](1))
    vb = s.computeVBPosterior(n, n)
    d = s.getDraws()
    w = vb["IS_weights"]
    assert np.all(w >= 0) and abs(w.sum() - 1) < 1e-12
    assert 1 <= 1 / np.sum(w ** 2) <= n
    k = 12
    th = np.asfortranarray(d["thetas"][:, :, :k].transpose(0, 2, 1))
    ld = oracle.logdet(wl["sp"], th)
    tol = 1e-10 if precision == "fp64" else 5e-4
    np.testing.assert_allclose(d["log_dets"][:k], ld, rtol=0, atol=tol)
    for key in ("m", "C", "n", "s"):  # finite even when the weights collapse
        assert np.all(np.isfinite(vb[key]))
    s.computePrior()
    x = wl["F_of"](2, False)
    out = s.computeForecastDebug(n, n, x)
    seed, epoch = 21, 1
    lam = np.asfortranarray(out["lambdas"][:, :k].T)
    th = np.asfortranarray(out["thetas"][:, :, :k].transpose(0, 2, 1))
    y, _ = oracle.forecast(wl["sp"], lam, th, x, seed, epoch)
    np.testing.assert_allclose(out["y"][:, :k], y, rtol=1e-5 if precision == "mixed" else 1e-9,
                               atol=1e-6 if precision == "mixed" else 1e-11)


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_diagonally_dominant_draws_stay_on_fast_path(built_lib, precision):
    """The benchmark's parental sets (m = 400) with |coefficients| <= 0.05 and a tight
    posterior: every (I - Gamma_i) is strictly diagonally dominant, so LU without
    pivoting is stable and the no-pivot pass must keep every draw (a flagged draw
    would still be right, through the pivoting redo, and so would hide a fault of
    the fast path); log|det| and forecasts against the oracle."""
    import bench

    wl = bench.make_workload(m=400, T=4, seed=11)
    m, P, n = wl["m"], wl["P"], 1024
    rng = np.random.default_rng(5)
    s = SGDLM(1, strict=True, precision=precision)
    s.setSimultaneousParents(wl["p"], np.where(wl["sp"] >= m * m, np.nan, wl["sp"]).astype(float))
    s.setDiscountFactors(np.full(m, 0.99), np.full((P, P, m), 0.99))
    mt = np.asfortranarray(rng.uniform(-0.05, 0.05, size=(P, m)))
    C = np.asfortranarray(np.repeat((1e-8 * np.eye(P))[:, :, None], m, axis=2))
    s.setPosteriorParameters(mt, C, np.full(m, 50.0), np.full(m, 1.0))
    s.setRngState(33, 0)
    s.computeVBPosterior(n, n)
    assert s.getStats()["draws_pivoted"] == 0
    d = s.getDraws()
    k = 16
    th = np.asfortranarray(d["thetas"][:, :, :k].transpose(0, 2, 1))
    ld = oracle.logdet(wl["sp"], th)
    np.testing.assert_allclose(d["log_dets"][:k], ld, rtol=0,
                               atol=1e-10 if precision == "fp64" else 1e-4)
    s.computePrior()
    x = wl["F_of"](2, False)
    out = s.computeForecastDebug(n, n, x)
    assert s.getStats()["draws_pivoted"] == 0
    lam = np.asfortranarray(out["lambdas"][:, :k].T)
    th = np.asfortranarray(out["thetas"][:, :, :k].transpose(0, 2, 1))
    y, _ = oracle.forecast(wl["sp"], lam, th, x, 33, 1)
    np.testing.assert_allclose(out["y"][:, :k], y, rtol=1e-5 if precision == "mixed" else 1e-9,
                               atol=1e-6 if precision == "mixed" else 1e-11)


@pytest.mark.parametrize("m", [40, 100, 150, 190, 224, 240, 300])
@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_dense_core_sizes(built_lib, precision, m):
    """No sparse levels, so the dense core is all m nodes: d_p = 64 .. 320 covers the
    panel schedules of the tensor-core LU (one 128-row tile from the start at
    d_p = 160, two tiles at 192 and 224) and the FFMA instantiation (d_p = 256, 320,
    where the panel Gauss-Jordan also hands rows beyond 224 to the separate
    multiplier GEMM).  Diagonally dominant draws: no draw may be redone with
    pivoting; log|det| and forecasts against the oracle."""
    import bench

    wl = bench.make_workload(m=m, T=4, seed=100 + m)
    P, n = wl["P"], 256
    rng = np.random.default_rng(m)
    s = SGDLM(1, strict=True, precision=precision)
    s.setSimultaneousParents(wl["p"], np.where(wl["sp"] >= m * m, np.nan, wl["sp"]).astype(float))
    s.setEliminationLevels(0)
    assert s.getEliminationInfo()["core_n"] == m
    s.setDiscountFactors(np.full(m, 0.99), np.full((P, P, m), 0.99))
    mt = np.asfortranarray(rng.uniform(-0.05, 0.05, size=(P, m)))
    C = np.asfortranarray(np.repeat((1e-8 * np.eye(P))[:, :, None], m, axis=2))
    s.setPosteriorParameters(mt, C, np.full(m, 50.0), np.full(m, 1.0))
    s.setRngState(44, 0)
    s.computeVBPosterior(n, n)
    assert s.getStats()["draws_pivoted"] == 0
    d = s.getDraws()
    k = 12
    th = np.asfortranarray(d["thetas"][:, :, :k].transpose(0, 2, 1))
    ld = oracle.logdet(wl["sp"], th)
    np.testing.assert_allclose(d["log_dets"][:k], ld, rtol=0,
                               atol=1e-10 if precision == "fp64" else 1e-4)
    s.computePrior()
    x = wl["F_of"](2, False)
    out = s.computeForecastDebug(n, n, x)
    assert s.getStats()["draws_pivoted"] == 0
    lam = np.asfortranarray(out["lambdas"][:, :k].T)
    th = np.asfortranarray(out["thetas"][:, :, :k].transpose(0, 2, 1))
    y, _ = oracle.forecast(wl["sp"], lam, th, x, 44, 1)
    # mixed: the oracle regenerates nu's normals in FP64, the GPU by FP32 Box-Muller
    # (absolute error ~1e-6); that error, carried through (I - Gamma)^-1, bounds the
    # agreement of the refined solves, hence the absolute term
    np.testing.assert_allclose(out["y"][:, :k], y, rtol=1e-5 if precision == "mixed" else 1e-9,
                               atol=5e-6 if precision == "mixed" else 1e-11)


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_all_draws_singular_give_nan_weights(built_lib, precision):
    """Two series, each the other's only parent, with coefficients exactly 1 and no
    posterior spread: every (I - Gamma_i) = [[1, -1], [-1, 1]] is singular.  The
    reference then divides 0 by 0 for every weight (SGDLM.cu:325-335); here the
    weights are NaN as well and sum |det| is 0 (the weights run over several
    blocks: n spans more than one)."""
    m, P, n = 2, 1, 700
    sp = np.array([[0 + 2 * 1, 1 + 2 * 0]], dtype=np.float64)  # 0 <- 1, 1 <- 0
    s = SGDLM(1, strict=True, precision=precision)
    s.setSimultaneousParents([1, 1], sp)
    s.setDiscountFactors(np.full(m, 0.95), np.full((P, P, m), 0.95))
    s.setPosteriorParameters(np.ones((P, m)), np.zeros((P, P, m)), np.full(m, 20.0),
                             np.full(m, 1.0))
    s.setRngState(3, 0)
    vb = s.computeVBPosterior(n, n)
    assert np.isnan(vb["IS_weights"]).all()
    assert vb["sum_det_weights"] == 0.0


def test_dag_parents_have_unit_determinant(built_lib):
    """Parents only among lower-indexed series: (I - Gamma) is unit lower triangular,
    det = 1 for every draw, the weights are uniform and ESS = n."""
    m, P, n = 300, 8, 512
    rng = np.random.default_rng(3)
    sp = np.full((P, m), np.nan)
    p = np.zeros(m, dtype=int)
    for j in range(m):
        k = min(j, int(rng.integers(0, 6)))
        pars = rng.choice(j, size=k, replace=False) if k else []
        p[j] = 2 + k
        for t, par in enumerate(pars):
            sp[2 + t, j] = j + m * par
    s = SGDLM(1, strict=True, precision="mixed")
    s.setSimultaneousParents(p, sp)
    s.setDiscountFactors(np.full(m, 0.95), np.full((P, P, m), 0.95))
    C = np.repeat((0.05 * np.eye(P))[:, :, None], m, axis=2)
    s.setPosteriorParameters(np.full((P, m), 0.1), C, np.full(m, 20.0), np.full(m, 0.01))
    vb = s.computeVBPosterior(n, n)
    d = s.getDraws()
    np.testing.assert_allclose(d["log_dets"], 0.0, atol=1e-5)
    np.testing.assert_allclose(vb["IS_weights"], 1.0 / n, rtol=1e-4)
