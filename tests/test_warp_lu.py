"""The warp-per-draw LU for small systems (m <= 32): log|det| of every draw and
the forecast solves against the oracle's FP64 partial-pivoting LU on the very
values the GPU drew, and against the block LU kernels on the same draws.

Tolerances: FP64 draws 1e-12 (log|det|, absolute) and 1e-10 (forecasts, normwise
per draw); FP32 draws: log|det| within the mixed form's gate of 1e-5 absolute,
forecasts (three refinements with an FP64 residual) within 1e-5 normwise (the
right-hand side itself carries the FP32 normals' ~1e-6)."""
import numpy as np
import pytest

import oracle
from gpusgdlm_gb300 import SGDLM

pytestmark = pytest.mark.gpu


def _model(m, kmax, precision, seed, warp=True):
    import bench

    wl = bench.make_workload(m=m, kmax=kmax, T=4, seed=seed)
    P = wl["P"]
    s = SGDLM(1, strict=True, precision=precision)
    s.setWarpLu(warp)
    s.setSimultaneousParents(wl["p"], np.where(wl["sp"] >= m * m, np.nan, wl["sp"]).astype(float))
    s.setDiscountFactors(np.full(m, 0.97), np.full((P, P, m), 0.98))
    rng = np.random.default_rng(seed)
    mt = np.asfortranarray(rng.normal(0.0, 0.15, size=(P, m)))
    C = np.asfortranarray(np.repeat((0.01 * np.eye(P))[:, :, None], m, axis=2))
    return s, wl, mt, C


def _spu(wl):
    return np.asarray(wl["sp"], dtype=np.uint32)


@pytest.mark.parametrize("m", [2, 6, 20, 32])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_warp_lu_logdet_and_forecast_vs_oracle(built_lib, precision, m):
    n = 1000
    s, wl, mt, C = _model(m, min(17, m - 1), precision, 100 + m)
    assert s.getWarpLu()["enabled"]
    s.setPosteriorParameters(mt, C, np.full(m, 20.0), np.full(m, 1.0))
    s.setRngState(7, 0)
    s.computeVBPosterior(n, n)
    assert s.getWarpLu()["in_use"]
    st = s.getStats()
    assert st["draws_pivoted"] == 0 and st["draws_singular"] == 0
    d = s.getDraws()
    th = np.asfortranarray(d["thetas"].transpose(0, 2, 1))
    ld = oracle.logdet(_spu(wl), th)
    err = np.abs(d["log_dets"] - ld).max()
    assert err <= (1e-5 if precision == "mixed" else 1e-12), err
    # forecasts
    P = wl["P"]
    x = np.asfortranarray(np.random.default_rng(m).normal(size=(P, m)))
    s.setPriorParameters(mt, C, np.full(m, 20.0), np.full(m, 1.0))
    s.setRngState(11, 0)
    out = s.computeForecastDebug(n, n, x)
    assert s.getStats()["forecast_draws_factored"] == n
    lam = np.asfortranarray(out["lambdas"].T)
    th = np.asfortranarray(out["thetas"].transpose(0, 2, 1))
    y, _ = oracle.forecast(_spu(wl), lam, th, x, 11, 0)
    e = (np.abs(out["y"] - y).max(axis=0) / np.abs(y).max(axis=0)).max()
    # FP32 draws: nu is summed in FP32 from FP32 normals (~1e-6 of the FP64 stream)
    assert e <= (1e-5 if precision == "mixed" else 1e-10), e
    s.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_warp_lu_equals_block_lu(built_lib, precision):
    """Same draws through the warp path and the block LU kernels (sparse levels,
    dense core, pivoting redo): log|det| within rounding of each other."""
    m, n = 24, 2000
    res = {}
    for warp in (True, False):
        s, wl, mt, C = _model(m, 17, precision, 5, warp=warp)
        s.setPosteriorParameters(mt, C, np.full(m, 20.0), np.full(m, 1.0))
        s.setRngState(3, 0)
        s.computeVBPosterior(n, n)
        assert s.getWarpLu()["in_use"] == warp
        res[warp] = s.getDraws()["log_dets"]
        s.close()
    np.testing.assert_allclose(res[True], res[False], rtol=0,
                               atol=2e-5 if precision == "mixed" else 1e-12)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_warp_lu_large_multiplier(built_lib, precision):
    """Parents 0<-1, 1<-0, 2<-0 with Gamma_01 = 1e5: the pivot order differs
    from the diagonal one; no redo pass exists on the warp path."""
    m, P = 3, 1
    sp = np.array([[0 + 3 * 1, 1 + 3 * 0, 2 + 3 * 0]], dtype=np.float64)
    s = SGDLM(1, strict=True, precision=precision)
    s.setSimultaneousParents([1, 1, 1], sp)
    s.setDiscountFactors(np.full(m, 0.95), np.full((P, P, m), 0.95))
    mt = np.array([[1.0e5, 20.0, -15.0]])
    C = np.full((1, 1, m), 1e-6)
    s.setPosteriorParameters(mt, C, np.full(m, 20.0), np.full(m, 1.0))
    s.setRngState(9, 0)
    s.computeVBPosterior(256, 256)
    assert s.getStats()["draws_pivoted"] == 0
    d = s.getDraws()
    th = np.asfortranarray(d["thetas"].transpose(0, 2, 1))
    spu = sp.astype(np.uint32)
    tol = dict(rtol=1e-6, atol=1e-6) if precision == "mixed" else dict(rtol=1e-13, atol=1e-13)
    np.testing.assert_allclose(d["log_dets"], oracle.logdet(spu, th), **tol)
    s.setPriorParameters(mt, C, np.full(m, 20.0), np.full(m, 1.0))
    s.setRngState(10, 0)
    x = np.zeros((P, m), order="F")
    out = s.computeForecastDebug(256, 256, x)
    lam = np.asfortranarray(out["lambdas"].T)
    th = np.asfortranarray(out["thetas"].transpose(0, 2, 1))
    y, _ = oracle.forecast(spu, lam, th, x, 10, 0)
    err = np.abs(out["y"] - y).max(axis=0) / np.abs(y).max(axis=0)
    assert err.max() <= (1e-5 if precision == "mixed" else 1e-11)
    s.close()


def test_warp_lu_not_used_above_32(built_lib):
    s, wl, mt, C = _model(33, 17, "mixed", 1)
    s.setPosteriorParameters(mt, C, np.full(33, 20.0), np.full(33, 1.0))
    s.computeVBPosterior(64, 64)
    assert s.getWarpLu() == {"enabled": True, "in_use": False}
    s.close()
