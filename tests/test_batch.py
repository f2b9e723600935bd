"""The batched multi-instance step (sgdlm_batch_*) and the LU tuner: engines of
different sizes advanced by one CUDA-graph launch per time step must equal the
same engines advanced one at a time (same kernels, same streams of random
numbers: bit for bit), before and after the autotuner has chosen their LU plans
and grids (which change the cost, not the arithmetic of a draw)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SIZES = [20, 33, 64, 100, 150, 230]


def _engine(m, seed):
    import bench
    from gpusgdlm_gb300 import SGDLM

    wl = bench.make_workload(m=m, kmax=min(17, m // 3), T=12, seed=seed)
    P = wl["P"]
    s = SGDLM(1, strict=True, precision="mixed")
    s.setSimultaneousParents(wl["p"], np.where(wl["sp"] >= m * m, np.nan, wl["sp"]).astype(float))
    s.setDiscountFactors(np.full(m, 0.97), np.full((P, P, m), 0.98))
    a, R, r, c = bench.prior_arrays(m, P)
    s.setPriorParameters(a, R, r, c)
    s.setRngState(1000 + seed, 0)
    return s, wl


class _Inputs:
    """Per-engine device buffers for (y, F, F_t+1) and the outputs."""

    def __init__(self, torch, wl, n):
        dev = torch.device("cuda:0")
        m, P = wl["m"], wl["P"]
        self.wl = wl
        self.y = torch.zeros(m, dtype=torch.float64, device=dev)
        self.F = torch.zeros(P * m, dtype=torch.float64, device=dev)
        self.x = torch.zeros(P * m, dtype=torch.float64, device=dev)
        self.fc = torch.zeros(n * m, dtype=torch.float64, device=dev)
        self.st = torch.zeros(8, dtype=torch.float64, device=dev)

    def load(self, torch, t):
        wl = self.wl
        self.y.copy_(torch.tensor(wl["y"][t]))
        self.F.copy_(torch.tensor(wl["F_of"](t).ravel(order="F")))
        self.x.copy_(torch.tensor(wl["F_of"](t + 1, False).ravel(order="F")))


def _setup(torch, n):
    from gpusgdlm_gb300 import Batch

    batched, single = [], []
    for k, m in enumerate(SIZES):
        sb, wl = _engine(m, 10 + k)
        ss, _ = _engine(m, 10 + k)
        for s in (sb, ss):
            s._ensure_sim(n, n)
        batched.append((sb, _Inputs(torch, wl, n)))
        single.append((ss, _Inputs(torch, wl, n)))
    b = Batch([s for s, _ in batched])
    b.record([io.y.data_ptr() for _, io in batched], [io.F.data_ptr() for _, io in batched],
             [io.x.data_ptr() for _, io in batched], n / 2.0,
             [io.fc.data_ptr() for _, io in batched], None, [io.st.data_ptr() for _, io in batched])
    return b, batched, single


def _advance(torch, b, batched, single, t0, t1, n):
    for t in range(t0, t1):
        for (_, io) in batched + single:
            io.load(torch, t)
        torch.cuda.synchronize()
        b.step()
        for s, io in single:
            assert s.filterStepDevice(io.y.data_ptr(), io.F.data_ptr(), io.x.data_ptr(), n / 2.0,
                                      io.fc.data_ptr(), None, io.st.data_ptr())
        for s, _ in batched + single:
            s.synchronize()


def _assert_equal(batched, single):
    for (sb, ib), (ss, is_) in zip(batched, single):
        pb, ps = sb.getParameters(), ss.getParameters()
        for k in ("m", "C", "n", "s"):
            np.testing.assert_array_equal(pb[k], ps[k])
        np.testing.assert_array_equal(ib.fc.cpu().numpy(), is_.fc.cpu().numpy())
        np.testing.assert_array_equal(ib.st.cpu().numpy(), is_.st.cpu().numpy())
        assert sb.getRngState() == ss.getRngState()


def test_batched_steps_equal_one_at_a_time(built_lib):
    torch = pytest.importorskip("torch")
    n = 2000
    b, batched, single = _setup(torch, n)
    _advance(torch, b, batched, single, 1, 5, n)
    _assert_equal(batched, single)
    b.close()


def test_autotuned_batch_equals_one_at_a_time_with_the_same_plans(built_lib):
    torch = pytest.importorskip("torch")
    n = 2000
    b, batched, single = _setup(torch, n)
    _advance(torch, b, batched, single, 1, 3, n)
    before = [s.getParameters() for s, _ in batched]
    tune = b.autotune(replays=2)
    assert tune["concurrency"] in (1, 2, 4, 8)
    assert tune["buckets"] == len({(m + 31) // 32 for m in SIZES})
    assert all(c > 0 for c in tune["ms_candidates"])
    # the trial steps were undone
    for (s, _), p0 in zip(batched, before):
        p1 = s.getParameters()
        for k in ("m", "C", "n", "s"):
            np.testing.assert_array_equal(p1[k], p0[k])
    # the same plans for the engines stepped one at a time
    for (sb, _), (ss, _) in zip(batched, single):
        o = sb.getLuOptions()
        ss.setLuOptions(o["allow_tensor_cores"], o["max_ctas"])
        ss.setEliminationLevels(sb.getEliminationInfo()["levels"])
        assert ss.getEliminationInfo() == sb.getEliminationInfo()
    _advance(torch, b, batched, single, 3, 6, n)
    _assert_equal(batched, single)
    b.close()


def test_tune_lu_keeps_results_within_rounding(built_lib):
    """The tuner's choice changes the cost, not the answer: log|det| of the same
    draws under the chosen plan equals the default plan's to FP32 rounding
    (diagonally dominant draws, so no draw changes between the fast pass and the
    pivoting pass)."""
    n = 1000
    s, wl = _engine(150, 3)
    m, P = wl["m"], wl["P"]
    rng = np.random.default_rng(4)
    mt = np.asfortranarray(rng.uniform(-0.05, 0.05, size=(P, m)))
    C = np.asfortranarray(np.repeat((1e-8 * np.eye(P))[:, :, None], m, axis=2))
    s.setPosteriorParameters(mt, C, np.full(m, 50.0), np.full(m, 1.0))
    s.setRngState(5, 0)
    s.computeVBPosterior(n, n)
    ld0 = s.getDraws()["log_dets"]
    t = s.tuneLu()
    assert t["ms"] > 0 and t["levels"] == s.getEliminationInfo()["levels"]
    assert min(c for c in t["ms_candidates"] if c > 0) == pytest.approx(t["ms"])
    s.setRngState(5, 0)
    s.computeVBPosterior(n, n)
    assert s.getStats()["draws_pivoted"] == 0
    ld1 = s.getDraws()["log_dets"]
    np.testing.assert_allclose(ld1, ld0, rtol=0, atol=1e-5)
    s.close()
