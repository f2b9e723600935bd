"""A CPU twin of the engine's state machine built from the oracle's stages.

Test infrastructure: it replays the same call sequence as the GB300 engine
(include/sgdlm.h) with the same Philox epochs, so that a GPU run and an oracle run
can be compared call by call.  Epoch rules (one epoch per sampling call):
computeVBPosterior, computeForecast (its draws and its nus), and each
evolveForecastSamples consume one epoch each.
"""
from __future__ import annotations

import numpy as np

import oracle


class OracleSGDLM:
    def __init__(self, p, sp, beta, delta, seed=1234, epoch=0, compat=3, nthreads=0):
        self.p = np.asarray(p, dtype=np.uint32)
        self.sp = np.asfortranarray(np.asarray(sp, dtype=np.uint32))
        self.beta = np.asarray(beta, dtype=np.float64)
        self.delta = np.asfortranarray(delta, dtype=np.float64)
        self.seed, self.epoch, self.compat, self.nthreads = seed, epoch, compat, nthreads
        P, m = self.sp.shape
        self.P, self.m = P, m
        self.W = np.zeros((P, P, m), order="F")

    def set_parameters(self, m_t, C_t, n_t, s_t):
        self.m_t = oracle.f64(m_t); self.C_t = oracle.f64(C_t)
        self.n_t = oracle.f64(n_t); self.s_t = oracle.f64(s_t)

    def posterior(self, y, F):
        self.m_t, self.C_t, self.n_t, self.s_t = oracle.posterior(
            self.p, self.m_t, self.C_t, self.n_t, self.s_t, y, F)

    def vb(self, n):
        lam, th, _ = oracle.sample(self.p, self.m_t, self.C_t, self.n_t, self.s_t, n, self.seed,
                                   self.epoch, self.nthreads)
        self.epoch += 1
        ld = oracle.logdet(self.sp, th, self.nthreads)
        w, s = oracle.weights(ld)
        out = oracle.vb(self.p, self.n_t, self.s_t, w, lam, th)
        out.update(IS_weights=w, sum_det_weights=s, log_dets=ld, lambdas=lam, thetas=th)
        return out

    def prior(self):
        self.C_t, self.n_t, self.W = oracle.prior(self.p, self.C_t, self.n_t, self.beta, self.delta,
                                                  self.W)

    def evo_prior(self, G):
        self.m_t, self.C_t, self.n_t, self.W = oracle.evo_prior(self.p, self.m_t, self.C_t, self.n_t,
                                                              self.beta, self.delta, G)

    def forecast(self, n, x, G4=None):
        """computeForecast for a P x m (one step) or P x m x K array (RcppWrapper.cpp:455-472);
        with evolution matrices G4 (P x P x m x KG) computeEvoForecast (:576-688)."""
        x = np.asarray(x, dtype=np.float64)
        K = 1 if x.ndim == 2 else x.shape[2]
        x3 = x.reshape(self.P, self.m, K, order="F")
        fm, fC, fn, fs, fW = self.m_t, self.C_t, self.n_t, self.s_t, self.W
        ys = []
        lam = th = None
        for k in range(K):
            if k == 0:
                lam, th, _ = oracle.sample(self.p, fm, fC, fn, fs, n, self.seed, self.epoch,
                                           self.nthreads)
            else:
                G = None if G4 is None else G4[:, :, :, k if G4.shape[3] > 1 else 0]
                lam, th, _ = oracle.evolve(self.p, fW, fn, fs, self.beta, lam, th, self.seed,
                                           self.epoch, self.compat, self.nthreads, G=G)
                self.epoch += 1
            y, _ = oracle.forecast(self.sp, lam, th, np.asfortranarray(x3[:, :, k]), self.seed,
                                   self.epoch, self.nthreads)
            self.epoch += 1
            ys.append(y)
        return ys[0] if x.ndim == 2 else np.stack(ys, axis=2)
