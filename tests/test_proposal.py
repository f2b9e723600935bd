"""The learned importance proposal: its network, density ratios, training and
fallback (gpusgdlm_gb300/csrc/mlp_kernels.cu, proposal_kernels.cu; oracle in
oracle/mlp.py).

CPU: the oracle's analytic gradient against central differences, and its
normal-gamma log density against scipy's distributions.
GPU (through the C ABI): the network's loss and gradients against the oracle
(BF16 weights on both sides, FP32 accumulation on the device: 2e-3 relative to
the gradient's scale); the importance weights of draws from a learned proposal
against the oracle's exact density ratios (FP64: 1e-9; mixed: 2e-4 absolute in
log weight); the IS moments of a perturbed proposal against the plain
proposal's within Monte-Carlo error; training, on posteriors whose VB refit
differs systematically from the naive one, lowering the loss and raising the
ESS over the plain proposal's; the ESS fallback.
"""
import numpy as np
import pytest

import oracle
from oracle import mlp as omlp

scipy_stats = pytest.importorskip("scipy.stats")


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(1)
    F, O, B = 9, 6, 7
    L = omlp.layout(F, O)
    w = (rng.normal(size=L["total"]) * 0.3).astype(np.float32)
    X = rng.normal(size=(B, F))
    Y = rng.normal(size=(B, O))
    M = (rng.uniform(size=(B, O)) > 0.2).astype(float)
    loss, g = omlp.loss_and_gradient(w, X, Y, M, F, O, round_bf16=False)
    w64 = w.astype(np.float64)
    idx = rng.choice(L["total"], size=40, replace=False)
    for k in idx:
        e = 1e-5

        def f(v):
            ww = w64.copy()
            ww[k] = v
            W1, b1, W2, b2, W3, b3 = [ww[a:b] for a, b in
                                      ((L["w1"], L["b1"]), (L["b1"], L["w2"]), (L["w2"], L["b2"]),
                                       (L["b2"], L["w3"]), (L["w3"], L["b3"]), (L["b3"], L["total"]))]
            Z1 = X @ W1.reshape(128, F).T + b1
            A2 = omlp.gelu(omlp.gelu(Z1) @ W2.reshape(128, 128).T + b2)
            out = A2 @ W3.reshape(O, 128).T + b3
            return (M * (out - Y) ** 2).sum() / M.sum()

        fd = (f(w64[k] + e) - f(w64[k] - e)) / (2 * e)
        assert abs(fd - g[k]) <= 1e-6 + 1e-5 * abs(fd), (k, fd, g[k])


def test_oracle_ng_logpdf_matches_scipy():
    rng = np.random.default_rng(2)
    for p in (0, 1, 3, 6):
        A = rng.normal(size=(p, p))
        C = A @ A.T + np.eye(p) * 0.5
        m = rng.normal(size=p)
        n, s = 7.3, 0.8
        lam = 1.7
        th = rng.normal(size=p)
        got = omlp.ng_logpdf(th, lam, m, C, n, s)
        ref = scipy_stats.gamma.logpdf(lam, a=n / 2, scale=2 / (n * s))
        if p:
            ref += scipy_stats.multivariate_normal.logpdf(th, mean=m, cov=C / (s * lam))
        assert abs(got - ref) < 1e-10


# ------------------------------------------------------------------ GPU tests
def _model(m, precision, seed=7, kmax=4):
    import bench
    from gpusgdlm_gb300 import SGDLM

    wl = bench.make_workload(m=m, kmax=kmax, T=60, seed=seed)
    P = wl["P"]
    s = SGDLM(1, strict=True, precision=precision)
    s.setSimultaneousParents(wl["p"], np.where(wl["sp"] >= m * m, np.nan, wl["sp"]).astype(float))
    s.setDiscountFactors(np.full(m, 0.97), np.full((P, P, m), 0.98))
    a, R, r, c = bench.prior_arrays(m, P)
    s.setPriorParameters(a, R, r, c)
    s.setRngState(11, 0)
    return s, wl


def _advance(s, wl, t0, t1, n):
    for t in range(t0, t1):
        s.computePosterior(wl["y"][t], wl["F_of"](t))
        vb = s.computeVBPosterior(n, n)
        if 1.0 / np.sum(vb["IS_weights"] ** 2) > n / 2:
            s.setPosteriorParameters(vb["m"], vb["C"], vb["n"], vb["s"])
        s.computePrior()


@pytest.mark.gpu
def test_network_loss_and_gradient_match_oracle(built_lib):
    s, wl = _model(12, "mixed")
    s.setProposal("learned", train_steps=5)
    nparam, F, O = s.proposalSizes()
    rng = np.random.default_rng(3)
    w = (rng.normal(size=nparam) * 0.2).astype(np.float32)
    s.setProposalParams(w)
    np.testing.assert_array_equal(s.getProposalParams(), w)
    B = 300
    X = rng.normal(size=(B, F)).astype(np.float32)
    Y = rng.normal(size=(B, O)).astype(np.float32)
    M = (rng.uniform(size=(B, O)) > 0.3).astype(np.float32)
    loss, g = s.proposalLossAndGradient(X, Y, M)
    ref_loss, ref_g = omlp.loss_and_gradient(w, X, Y, M, F, O)
    assert abs(loss - ref_loss) <= 1e-4 * abs(ref_loss)
    L = omlp.layout(F, O)
    for a, b in (("w1", "b1"), ("b1", "w2"), ("w2", "b2"), ("b2", "w3"), ("w3", "b3"), ("b3", "total")):
        gg, rr = g[L[a]:L[b]], ref_g[L[a]:L[b]]
        scale = np.max(np.abs(rr))
        assert np.max(np.abs(gg - rr)) <= 2e-3 * scale, (a, np.max(np.abs(gg - rr)), scale)
    s.close()


def _perturb_last_layer(s, scale, seed=5):
    nparam, F, O = s.proposalSizes()
    w = s.getProposalParams()
    L = omlp.layout(F, O)
    rng = np.random.default_rng(seed)
    w[L["w3"]:L["b3"]] = (rng.normal(size=L["b3"] - L["w3"]) * scale).astype(np.float32)
    w[L["b3"]:] = (rng.normal(size=O) * scale).astype(np.float32)
    s.setProposalParams(w)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_learned_weights_are_exact_density_ratios(built_lib, precision):
    """Draws from a perturbed learned proposal: every draw's log weight equals
    log|det(I - Gamma)| + sum_j [log p_j - log q_j] computed by the oracle from
    the device's own draws and the proposal's parameters."""
    m, n = 10, 400
    s, wl = _model(m, precision)
    _advance(s, wl, 1, 6, 2000)
    s.setProposal("learned", train_steps=0, ess_fraction=0.0)
    _perturb_last_layer(s, 0.05)
    s.computePosterior(wl["y"][6], wl["F_of"](6))
    post = s.getParameters()
    s.computeVBPosterior(n, n)
    info = s.getProposalInfo()
    assert info["used_learned"] == 1 and info["learned_calls"] == 1
    st = s.getProposalState()
    d = s.getDraws()
    p = wl["p"]
    lam, th = d["lambdas"], d["thetas"]            # (m, n), (P, m, n)
    ld = oracle.logdet(wl["sp"], np.asfortranarray(th.transpose(0, 2, 1)))
    ref = ld.copy()
    for i in range(n):
        for j in range(m):
            k = int(p[j])
            lp = omlp.ng_logpdf(th[:k, j, i], lam[j, i], post["m"][:k, j], post["C"][:k, :k, j],
                                post["n"][j], post["s"][j])
            lq = omlp.ng_logpdf(th[:k, j, i], lam[j, i], st["m"][:k, j], st["C"][:k, :k, j],
                                st["n"][j], st["s"][j])
            ref[i] += lp - lq
    tol = 1e-9 if precision == "fp64" else 2e-4
    np.testing.assert_allclose(st["log_weights"], ref, rtol=0, atol=tol * max(1.0, np.abs(ref).max()))
    # the proposal differs from the naive posterior
    assert np.max(np.abs(st["m"] - post["m"])) > 0
    s.close()


def _constant_outputs(s, delta, rho, a, b):
    """Network parameters whose outputs are the constants given (W3 = 0)."""
    nparam, F, O = s.proposalSizes()
    P = (O - 2) // 2
    w = s.getProposalParams()
    L = omlp.layout(F, O)
    w[L["w3"]:L["b3"]] = 0.0
    b3 = np.zeros(O, dtype=np.float32)
    b3[:P], b3[P:2 * P], b3[2 * P], b3[2 * P + 1] = delta, rho, a, b
    w[L["b3"]:] = b3
    s.setProposalParams(w)


@pytest.mark.gpu
def test_learned_proposal_moments_agree_with_plain_within_mc_error(built_lib):
    """A consistent estimator: the VB moments under a learned proposal (shifted
    by 0.1 sd, 20 % wider, a gamma of smaller shape: heavier tails than the
    target, so the weights have finite variance) and under the plain proposal
    agree within Monte-Carlo error (FP64, 12 replicates each)."""
    m, n, K = 10, 4000, 12
    s, wl = _model(m, "fp64")
    _advance(s, wl, 1, 6, 2000)
    s.computePosterior(wl["y"][6], wl["F_of"](6))
    post = s.getParameters()

    def runs():
        out = []
        for k in range(K):
            s.setPosteriorParameters(post["m"], post["C"], post["n"], post["s"])
            s.setRngState(100 + k, 0)
            vb = s.computeVBPosterior(n, n)
            out.append(np.concatenate([vb["m"].ravel(), vb["n"], vb["s"]]))
        return np.array(out)

    plain = runs()
    s.setProposal("learned", train_steps=0, ess_fraction=0.0)
    _constant_outputs(s, 0.1, 0.2, -0.2, 0.0)
    learned = runs()
    assert s.getProposalInfo()["learned_calls"] == K
    mu_p, mu_l = plain.mean(0), learned.mean(0)
    se = np.sqrt(plain.var(0, ddof=1) / K + learned.var(0, ddof=1) / K)
    ok = se > 0
    z = (mu_l[ok] - mu_p[ok]) / se[ok]
    print("z:", np.round(np.sort(np.abs(z))[-5:], 2))
    assert np.mean(np.abs(z) < 3) >= 0.95 and np.max(np.abs(z)) < 6
    s.close()


def _coupled_pairs(precision="mixed", seed=5):
    """Five pairs of series, each the other's simultaneous parent with a
    coefficient of mean 0.8 and sd 0.1: |det(I - Gamma)| = prod |1 - g_a g_b|
    varies strongly across draws, so the VB refit moves the coefficients'
    posterior systematically away from the naive one."""
    from gpusgdlm_gb300 import SGDLM

    m, P = 10, 2
    sp = np.full((P, m), np.nan)
    for j in range(m):
        sp[1, j] = j + m * (j ^ 1)
    s = SGDLM(1, strict=True, precision=precision)
    s.setSimultaneousParents(np.full(m, 2), sp)
    s.setDiscountFactors(np.full(m, 0.97), np.full((P, P, m), 0.98))
    mt = np.zeros((P, m), order="F")
    mt[1, :] = 0.8
    C = np.repeat(np.diag([0.01, 0.01])[:, :, None], m, axis=2)
    state = (mt, C, np.full(m, 30.0), np.full(m, 1.0))
    s.setRngState(seed, 0)
    return s, state


@pytest.mark.gpu
def test_training_learns_the_vb_shift_and_raises_ess(built_lib):
    """Online training on (naive -> VB) pairs where the VB refit differs
    systematically from the naive posterior: the loss falls to the refit's
    Monte-Carlo noise, the deployed proposal sits closer to the VB refit than the
    naive posterior, and its importance weights have a higher ESS than the plain
    proposal's at the same posterior -- what the network gains."""
    n = 4000
    s, state = _coupled_pairs()
    s.setProposal("learned", train_steps=30, iters_per_step=16, batch=256, lr=3e-3)
    losses = []
    for k in range(30):
        s.setPosteriorParameters(*state)
        vb = s.computeVBPosterior(n, n)
        losses.append(s.getProposalInfo()["last_loss"])
    info = s.getProposalInfo()
    assert info["deployed"] == 1 and info["training_calls"] == 30
    print("loss first/last:", losses[:3], losses[-3:])
    assert np.mean(losses[-5:]) < 0.5 * np.mean(losses[:5])
    plain, _ = _coupled_pairs(seed=6)
    ess_l, ess_p, d_l, d_p = [], [], [], []
    for k in range(8):
        s.setPosteriorParameters(*state)
        vb = s.computeVBPosterior(n, n)
        i = s.getProposalInfo()
        assert i["used_learned"] == 1
        ess_l.append(i["ess_learned"])
        q = s.getProposalState()
        plain.setPosteriorParameters(*state)
        pv = plain.computeVBPosterior(n, n)
        ess_p.append(1.0 / np.sum(pv["IS_weights"] ** 2))
        d_l.append(np.sum((q["m"][1] - pv["m"][1]) ** 2))
        d_p.append(np.sum((state[0][1] - pv["m"][1]) ** 2))
    print("ESS learned / plain:", np.mean(ess_l), np.mean(ess_p))
    assert np.mean(d_l) < np.mean(d_p)
    assert np.mean(ess_l) > 1.05 * np.mean(ess_p)
    s.close()
    plain.close()


@pytest.mark.gpu
def test_low_ess_falls_back_to_plain_proposal(built_lib):
    """A proposal far from the posterior gives a low ESS: the call is redone with
    the plain proposal and reports it."""
    m, n = 10, 1000
    s, wl = _model(m, "mixed")
    _advance(s, wl, 1, 6, 2000)
    s.setProposal("learned", train_steps=0, ess_fraction=0.5)
    nparam, F, O = s.proposalSizes()
    w = s.getProposalParams()
    L = omlp.layout(F, O)
    P = (O - 2) // 2
    b3 = np.zeros(O, dtype=np.float32)
    b3[:P] = 3.0  # location shifts of 3 sd on every coefficient
    w[L["b3"]:] = b3
    s.setProposalParams(w)
    s.computePosterior(wl["y"][6], wl["F_of"](6))
    vb = s.computeVBPosterior(n, n)
    info = s.getProposalInfo()
    assert info["learned_calls"] == 1 and info["fallbacks"] == 1 and info["used_learned"] == 0
    assert info["ess_learned"] < 0.5 * n and info["ess_plain"] > 0.5 * n
    assert abs(1.0 / np.sum(vb["IS_weights"] ** 2) - info["ess_plain"]) < 1e-6 * n
    s.close()
