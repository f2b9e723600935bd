"""CPU oracle of the learned importance proposal -- TEST INFRASTRUCTURE ONLY.

The reference has no learned proposal (its proposal is the decoupled naive
posterior, rSGDLM/src/SGDLM/SGDLM.cu:623-677); this module restates, in plain
numpy FP64, what gpusgdlm_gb300/csrc/mlp_kernels.cu and proposal_kernels.cu
compute, so that the tests can check the CUDA path:

* the network features -> 128 -> GELU -> 128 -> GELU -> outputs with BF16
  weights (rounded to nearest even, as the kernels' copies), its masked MSE and
  the gradient of every parameter (the flat FP32 layout of include/sgdlm.h);
* the normal-gamma log density NG(theta, lambda | m, C, n, s) =
  Gamma(lambda | n/2, rate n s/2) N(theta | m, C / (s lambda)) and the proposal
  the network's outputs define.
Only tests/ and bench.py's CPU legs may import it.
"""
from __future__ import annotations

import math

import numpy as np
from scipy.special import erf, gammaln

H = 128
DELTA_MAX, RHO_MAX, SHAPE_MAX = 3.0, 1.0, 2.0


def layout(F, O):
    w1 = 0
    b1 = w1 + H * F
    w2 = b1 + H
    b2 = w2 + H * H
    w3 = b2 + H
    b3 = w3 + O * H
    return dict(F=F, O=O, w1=w1, b1=b1, w2=w2, b2=b2, w3=w3, b3=b3, total=b3 + O)


def bf16(x):
    """Round FP32 values to BF16 (nearest, ties to even), returned as float64."""
    a = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = ((a + 0x7FFF + ((a >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(w, F, O, round_bf16=True):
    L = layout(F, O)
    w = np.asarray(w, dtype=np.float32)
    cvt = bf16 if round_bf16 else (lambda v: np.asarray(v, dtype=np.float64))
    W1 = cvt(w[L["w1"]:L["b1"]]).reshape(H, F)
    W2 = cvt(w[L["w2"]:L["b2"]]).reshape(H, H)
    W3 = cvt(w[L["w3"]:L["b3"]]).reshape(O, H)
    b1 = w[L["b1"]:L["w2"]].astype(np.float64)
    b2 = w[L["b2"]:L["w3"]].astype(np.float64)
    b3 = w[L["b3"]:L["total"]].astype(np.float64)
    return W1, b1, W2, b2, W3, b3


def gelu(x):
    return 0.5 * x * (1.0 + erf(x / math.sqrt(2.0)))


def gelu_grad(x):
    return 0.5 * (1.0 + erf(x / math.sqrt(2.0))) + x * np.exp(-0.5 * x * x) / math.sqrt(2 * math.pi)


def forward(w, X, F, O, round_bf16=True):
    W1, b1, W2, b2, W3, b3 = unpack(w, F, O, round_bf16)
    X = np.asarray(X, dtype=np.float64)
    Z1 = X @ W1.T + b1
    A1 = gelu(Z1)
    Z2 = A1 @ W2.T + b2
    A2 = gelu(Z2)
    return A2 @ W3.T + b3, (X, Z1, A1, Z2, A2)


def loss_and_gradient(w, X, Y, mask, F, O, round_bf16=True):
    """Masked MSE sum(mask (out - Y)^2) / sum(mask) and its gradient (flat)."""
    W1, b1, W2, b2, W3, b3 = unpack(w, F, O, round_bf16)
    out, (X, Z1, A1, Z2, A2) = forward(w, X, F, O, round_bf16)
    Y = np.asarray(Y, dtype=np.float64)
    M = np.asarray(mask, dtype=np.float64)
    cnt = max(M.sum(), 1.0)
    loss = float((M * (out - Y) ** 2).sum() / cnt)
    dO = 2.0 * M * (out - Y) / cnt
    g3, gb3 = dO.T @ A2, dO.sum(0)
    dZ2 = (dO @ W3) * gelu_grad(Z2)
    g2, gb2 = dZ2.T @ A1, dZ2.sum(0)
    dZ1 = (dZ2 @ W2) * gelu_grad(Z1)
    g1, gb1 = dZ1.T @ X, dZ1.sum(0)
    L = layout(F, O)
    g = np.zeros(L["total"])
    g[L["w1"]:L["b1"]] = g1.ravel()
    g[L["b1"]:L["w2"]] = gb1
    g[L["w2"]:L["b2"]] = g2.ravel()
    g[L["b2"]:L["w3"]] = gb2
    g[L["w3"]:L["b3"]] = g3.ravel()
    g[L["b3"]:] = gb3
    return loss, g


def ng_logpdf(theta, lam, m, C, n, s):
    """log NG(theta, lambda | m, C, n, s) over the active coefficients (len(m))."""
    p = len(m)
    lg = 0.5 * n * math.log(0.5 * n * s) - gammaln(0.5 * n) + (0.5 * n - 1) * math.log(lam) \
        - 0.5 * n * s * lam
    if p == 0:
        return lg
    Cs = np.asarray(C, dtype=np.float64) / (s * lam)
    d = np.asarray(theta, dtype=np.float64) - m
    sign, logdet = np.linalg.slogdet(Cs)
    quad = d @ np.linalg.solve(Cs, d)
    return lg - 0.5 * (p * math.log(2 * math.pi) + logdet + quad)


def proposal(out, m_t, C_t, n_t, s_t, p):
    """The proposal (m~, C~, n~, s~) of one series from the network's outputs
    (2P + 2: delta, rho, a, b), as gpusgdlm_gb300/csrc/proposal_kernels.cu forms it."""
    P = len(m_t)
    pj = int(p)
    o = np.asarray(out, dtype=np.float64)
    dl = np.clip(o[:P], -DELTA_MAX, DELTA_MAX)
    rh = np.clip(o[P:2 * P], -RHO_MAX, RHO_MAX)
    dl[pj:] = 0.0
    rh[pj:] = 0.0
    sd = np.sqrt(np.diag(C_t))
    mq = m_t + dl * sd
    D = np.exp(rh)
    Cq = C_t * np.outer(D, D)
    nq = n_t * math.exp(float(np.clip(o[2 * P], -SHAPE_MAX, SHAPE_MAX)))
    sq = s_t * math.exp(float(np.clip(o[2 * P + 1], -SHAPE_MAX, SHAPE_MAX)))
    return mq, Cq, nq, sq
