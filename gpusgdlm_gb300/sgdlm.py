"""The ``SGDLM`` class: the reference's Rcpp module surface over the GB300 engine.

Method names, argument order, array shapes (R column-major) and return values
follow rSGDLM's ``SGDLM`` class (rSGDLM/src/R_main.cpp:16-39, implemented in
rSGDLM/src/SGDLM/RcppWrapper.cpp).  As there, a call with wrong dimensions or in
the wrong prior/posterior state logs an error and does nothing (it returns None;
``last_status`` holds the C status code).  ``SGDLM(strict=True)`` raises
``SGDLMError`` instead.

R's ``NA`` in the simultaneous-parent matrix ``sp`` may be given as ``NaN``,
``None``, a negative number or any value >= m*m; it is stored as the unsigned
value 2147483648, as the reference stores R's NA_integer_.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional

import numpy as np

from . import _lib as L

NA_UNSIGNED = 2147483648


class SGDLMError(RuntimeError):
    pass


def _f64(a, shape=None):
    arr = np.asfortranarray(np.asarray(a, dtype=np.float64))
    if shape is not None and arr.shape != shape:
        raise ValueError(f"expected shape {shape}, got {arr.shape}")
    return arr


def _pd(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_double))


def _pu(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_uint))


def encode_sp(sp, m: int) -> np.ndarray:
    """R integer matrix with NA -> unsigned P x m array (memory_manager_RCPP.hpp:31-45)."""
    a = np.asarray(sp, dtype=object)
    if a.ndim != 2:
        raise ValueError("sp must be a 2-D (max_p x m) array")
    out = np.empty(a.shape, dtype=np.uint32, order="F")
    for idx, v in np.ndenumerate(a):
        if v is None or (isinstance(v, float) and np.isnan(v)):
            out[idx] = NA_UNSIGNED
        else:
            iv = int(v)
            out[idx] = NA_UNSIGNED if iv < 0 or iv >= m * m else iv
    return out


class SGDLM:
    """Simultaneous Graphical DLM filter on one GB300 (rSGDLM's ``SGDLM``)."""

    def __init__(self, no_gpus: int = 1, strict: bool = False,
                 precision: str = "mixed", compat: int = L.COMPAT_REFERENCE):
        self._lib = L.lib()
        h = C.c_void_p()
        st = self._lib.sgdlm_create(int(no_gpus), C.byref(h))
        if st != L.OK:
            raise SGDLMError(f"sgdlm_create failed: {L.STATUS.get(st, st)}")
        self._h = h
        self.strict = strict
        self.last_status = L.OK
        self.setPrecision(precision)
        self._lib.sgdlm_set_compat(self._h, int(compat))

    # ------------------------------------------------------------ plumbing
    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                self._lib.sgdlm_destroy(h)
            except Exception:
                pass
            self._h = C.c_void_p()

    def close(self):
        self.__del__()

    def _check(self, st: int) -> bool:
        self.last_status = st
        if st != L.OK:
            if self.strict:
                msg = self._lib.sgdlm_last_error(self._h)
                raise SGDLMError(f"{L.STATUS.get(st, st)}: {msg.decode() if msg else ''}")
            return False
        return True

    def _bad_dim(self, msg: str):
        # RcppWrapper's dimension checks log and return (RcppWrapper.cpp:80-92)
        import sys
        print(f"Error: {msg}", file=sys.stderr)
        self.last_status = 1
        if self.strict:
            raise SGDLMError(f"SGDLM_ERR_BAD_DIM: {msg}")
        return None

    def _size(self, fn) -> int:
        v = C.c_size_t()
        fn(self._h, C.byref(v))
        return int(v.value)

    @property
    def m(self) -> int:
        return self._size(self._lib.sgdlm_get_no_series)

    @property
    def max_p(self) -> int:
        return self._size(self._lib.sgdlm_get_max_p)

    @property
    def nsim(self) -> int:
        return self._size(self._lib.sgdlm_get_nsim)

    @property
    def nsim_batch(self) -> int:
        return self._size(self._lib.sgdlm_get_nsim_batch)

    # ------------------------------------------------- parental structure
    def getSimultaneousParents(self):
        """RcppWrapper.cpp:46-71 -> {'p', 'sp'}; NA entries of sp are NaN."""
        m, P = self.m, self.max_p
        p = np.zeros(m, dtype=np.uint32)
        sp = np.zeros((P, m), dtype=np.uint32, order="F")
        if not self._check(self._lib.sgdlm_get_parental_sets(self._h, _pu(p), _pu(sp))):
            return None
        spf = sp.astype(np.float64)
        spf[sp >= m * m] = np.nan
        return {"p": p.astype(np.int64), "sp": spf}

    def setSimultaneousParents(self, p, sp):
        """RcppWrapper.cpp:73-121: (re)initialises device memory when m or max_p change."""
        sp_arr = np.asarray(sp, dtype=object)
        if sp_arr.ndim != 2:
            return self._bad_dim("Incorrect dimension of sp")
        p = np.asarray(p, dtype=np.int64).ravel()
        P, m = sp_arr.shape
        if len(p) != m:
            return self._bad_dim("Dimensions of input arguments are incompatible")
        if self.m != m or self.max_p != P:
            if not self._check(self._lib.sgdlm_init_memory(self._h, m, P)):
                return None
        pu = np.ascontiguousarray(p.astype(np.uint32))
        spu = encode_sp(sp_arr, m)
        self._check(self._lib.sgdlm_set_parental_sets(self._h, _pu(pu), _pu(spu)))
        return None

    # ---------------------------------------------------- discount factors
    def getDiscountFactors(self):
        m, P = self.m, self.max_p
        beta = np.zeros(m)
        delta = np.zeros((P, P, m), order="F")
        if not self._check(self._lib.sgdlm_get_discount_factors(self._h, _pd(beta), _pd(delta))):
            return None
        return {"beta": beta, "delta": delta}

    def setDiscountFactors(self, beta, Delta):
        """RcppWrapper.cpp:150-183."""
        m, P = self.m, self.max_p
        D = np.asarray(Delta)
        if D.ndim != 3:
            return self._bad_dim("Incorrect dimension of delta")
        beta = np.asarray(beta, dtype=np.float64).ravel()
        if len(beta) != m or D.shape != (P, P, m):
            return self._bad_dim("Dimensions of input arguments are incompatible")
        b, d = np.ascontiguousarray(beta), _f64(D)
        self._check(self._lib.sgdlm_set_discount_factors(self._h, _pd(b), _pd(d)))
        return None

    # ------------------------------------------------------------ parameters
    def getParameters(self):
        """RcppWrapper.cpp:185-219 -> {'m', 'C', 'n', 's'}."""
        m, P = self.m, self.max_p
        mt = np.zeros((P, m), order="F"); Ct = np.zeros((P, P, m), order="F")
        nt = np.zeros(m); st = np.zeros(m)
        if not self._check(self._lib.sgdlm_get_parameters(self._h, _pd(mt), _pd(Ct), _pd(nt), _pd(st))):
            return None
        return {"m": mt, "C": Ct, "n": nt, "s": st}

    def _set_parameters(self, m_t, C_t, n_t, s_t, is_prior: bool):
        """RcppWrapper.cpp:239-283."""
        m, P = self.m, self.max_p
        a1, a2 = np.asarray(m_t), np.asarray(C_t)
        if a1.ndim != 2 or a2.ndim != 3:
            return self._bad_dim("Incorrect dimension of the input arguments")
        n_t = np.asarray(n_t, dtype=np.float64).ravel()
        s_t = np.asarray(s_t, dtype=np.float64).ravel()
        if a1.shape != (P, m) or a2.shape != (P, P, m) or len(n_t) != m or len(s_t) != m:
            return self._bad_dim("Dimensions of input arguments are incompatible")
        a1, a2 = _f64(a1), _f64(a2)
        n_t, s_t = np.ascontiguousarray(n_t), np.ascontiguousarray(s_t)
        if self._check(self._lib.sgdlm_set_parameters(self._h, _pd(a1), _pd(a2), _pd(n_t), _pd(s_t))):
            self._lib.sgdlm_set_is_prior(self._h, 1 if is_prior else 0)
        return None

    def setPriorParameters(self, a, R, r, c):
        return self._set_parameters(a, R, r, c, True)

    def setPosteriorParameters(self, m_t, C_t, n_t, s_t):
        return self._set_parameters(m_t, C_t, n_t, s_t, False)

    def isPrior(self) -> bool:
        v = C.c_int()
        self._lib.sgdlm_is_prior(self._h, C.byref(v))
        return bool(v.value)

    # ------------------------------------------------------------- filtering
    def computePosterior(self, y_t, F_t):
        """RcppWrapper.cpp:285-314."""
        m, P = self.m, self.max_p
        F = np.asarray(F_t)
        if F.ndim != 2:
            return self._bad_dim("Incorrect dimension of the input arguments")
        y = np.asarray(y_t, dtype=np.float64).ravel()
        if len(y) != m or F.shape != (P, m):
            return self._bad_dim("Dimensions of input arguments are incompatible")
        y, F = np.ascontiguousarray(y), _f64(F)
        self._check(self._lib.sgdlm_compute_posterior(self._h, _pd(y), _pd(F)))
        return None

    def _ensure_sim(self, nsim: int, nsim_batch: int) -> bool:
        # RcppWrapper.cpp:322-325: re-initialise when (nsim, nsim_batch) change
        if nsim != self.nsim or nsim_batch != self.nsim_batch:
            return self._check(self._lib.sgdlm_init_sim_memory(self._h, int(nsim), int(nsim_batch)))
        return True

    def computeVBPosterior(self, nsim: int, nsim_batch: int):
        """RcppWrapper.cpp:316-369 -> {'m','C','n','s','IS_weights','sum_det_weights'}."""
        if not self._ensure_sim(nsim, nsim_batch):
            return None
        m, P, n = self.m, self.max_p, self.nsim
        mt = np.zeros((P, m), order="F"); Ct = np.zeros((P, P, m), order="F")
        nt = np.zeros(m); st = np.zeros(m); w = np.zeros(n); sw = C.c_double()
        if not self._check(self._lib.sgdlm_compute_vb_posterior(
                self._h, _pd(mt), _pd(Ct), _pd(nt), _pd(st), _pd(w), C.byref(sw))):
            return None
        return {"m": mt, "C": Ct, "n": nt, "s": st, "IS_weights": w,
                "sum_det_weights": float(sw.value)}

    def computePrior(self):
        """RcppWrapper.cpp:371-375."""
        self._check(self._lib.sgdlm_compute_prior(self._h, 0))
        return None

    def computeEvoPrior(self, G_tp1):
        """RcppWrapper.cpp:377-409: the prior step with an evolution matrix G_tp1
        (max_p x max_p x m): a = G m and R = G R G' after the discount."""
        m, P = self.m, self.max_p
        G = np.asarray(G_tp1, dtype=np.float64)
        if G.ndim != 3:
            return self._bad_dim("Incorrect dimension of the input arguments")
        if G.shape != (P, P, m):
            return self._bad_dim("Dimensions of input arguments are incompatible")
        G = np.asfortranarray(G)
        if not self._check(self._lib.sgdlm_manage_evo_memory(self._h, 1)):  # RcppWrapper.cpp:406
            return None
        self._check(self._lib.sgdlm_compute_evo_prior(self._h, _pd(G), 0))
        return None

    def getEvolutionMatrixConfiguration(self) -> bool:
        """HostWrapper.hpp:19: whether evolution matrices are enabled."""
        v = C.c_int()
        self._lib.sgdlm_get_evolution_matrix_configuration(self._h, C.byref(v))
        return bool(v.value)

    def manageEvoMemory(self, use_state_evolution_matrix: bool):
        """HostWrapper.hpp:31: enable or disable the evolution matrices."""
        self._check(self._lib.sgdlm_manage_evo_memory(self._h, 1 if use_state_evolution_matrix else 0))

    def getEvolutionMatrix(self):
        """HostWrapper.hpp:57: the current evolution matrices (max_p x max_p x m)."""
        m, P = self.m, self.max_p
        G = np.zeros((P, P, m), order="F")
        if not self._check(self._lib.sgdlm_get_evolution_matrix(self._h, _pd(G))):
            return None
        return G

    def setEvolutionMatrix(self, G_t):
        """HostWrapper.hpp:59: sets the evolution matrices (max_p x max_p x m)."""
        m, P = self.m, self.max_p
        G = np.asarray(G_t, dtype=np.float64)
        if G.shape != (P, P, m):
            return self._bad_dim("Dimensions of input arguments are incompatible")
        G = np.asfortranarray(G)
        self._check(self._lib.sgdlm_set_evolution_matrix(self._h, _pd(G)))
        return None

    def computeEvoForecast(self, nsim: int, nsim_batch: int, F_tp1, G_tp1):
        """RcppWrapper.cpp:576-688: multi-step forecast whose draws evolve with the
        evolution matrices G_tp1 (max_p x max_p x m, or x K with one matrix per
        step; a single matrix serves every step)."""
        m, P = self.m, self.max_p
        F = np.asarray(F_tp1, dtype=np.float64)
        if F.ndim not in (2, 3):
            return self._bad_dim("Incorrect dimension of the input arguments")
        if F.shape[0] != P or F.shape[1] != m:
            return self._bad_dim("Dimensions of input arguments are incompatible")
        K = 1 if F.ndim == 2 else F.shape[2]
        G = np.asarray(G_tp1, dtype=np.float64)
        if G.ndim not in (3, 4):
            return self._bad_dim("Incorrect dimension of the input arguments")
        KG = 1 if G.ndim == 3 else G.shape[3]
        if KG > 1 and KG != K:
            return self._bad_dim("Dimensions of input arguments are incompatible")
        if G.shape[0] != P or G.shape[1] != P or G.shape[2] != m:
            return self._bad_dim("Dimensions of input arguments are incompatible")
        G4 = np.asfortranarray(G.reshape(P, P, m, KG, order="F"))
        return self._forecast(nsim, nsim_batch, F_tp1, debug=False, G4=G4)

    def _forecast(self, nsim, nsim_batch, F_tp1, debug: bool, G4=None):
        """RcppWrapper.cpp:411-479 (and :481-574 for the debug variant; :576-688 with
        evolution matrices G4, max_p x max_p x m x KG)."""
        m, P = self.m, self.max_p
        F = np.asarray(F_tp1, dtype=np.float64)
        if F.ndim not in (2, 3):
            return self._bad_dim("Incorrect dimension of the input arguments")
        if F.shape[0] != P or F.shape[1] != m:
            return self._bad_dim("Dimensions of input arguments are incompatible")
        K = 1 if F.ndim == 2 else F.shape[2]
        if not self._ensure_sim(nsim, nsim_batch):
            return None
        n = self.nsim
        F3 = np.asfortranarray(F.reshape(P, m, K, order="F"))
        y = np.zeros((m, n, K), order="F")
        lam = np.zeros((m, n, K), order="F") if debug else None
        th = np.zeros((P, m, n, K), order="F") if debug else None
        if G4 is not None and not self._check(self._lib.sgdlm_manage_evo_memory(self._h, 1)):
            return None  # RcppWrapper.cpp:649
        if not self._check(self._lib.sgdlm_init_forecast_priors(self._h)):
            return None
        for k in range(K):
            if k > 0 and G4 is not None:
                Gk = np.asfortranarray(G4[:, :, :, k if G4.shape[3] > 1 else 0])
                if not self._check(self._lib.sgdlm_evolve_forecast_samples_evo(self._h, _pd(Gk))):
                    return None
            elif k > 0 and not self._check(self._lib.sgdlm_evolve_forecast_samples(self._h)):
                return None
            xk = np.asfortranarray(F3[:, :, k])
            yk = np.zeros((m, n), order="F")
            lk = np.zeros((m, n), order="F") if debug else None
            tk = np.zeros((P, m, n), order="F") if debug else None
            if not self._check(self._lib.sgdlm_compute_forecast(
                    self._h, _pd(yk), _pd(xk), _pd(lk), _pd(tk), 1 if k > 0 else 0)):
                return None
            y[:, :, k] = yk
            if debug:
                lam[:, :, k] = lk
                th[:, :, :, k] = tk
        if F.ndim == 2:
            y = y[:, :, 0]
            if debug:
                lam, th = lam[:, :, 0], th[:, :, :, 0]
        if debug:
            return {"y": y, "lambdas": lam, "thetas": th}
        return y

    def computeForecast(self, nsim: int, nsim_batch: int, F_tp1):
        return self._forecast(nsim, nsim_batch, F_tp1, debug=False)

    def computeForecastDebug(self, nsim: int, nsim_batch: int, F_tp1):
        return self._forecast(nsim, nsim_batch, F_tp1, debug=True)

    # -------------------------------------------------------- memory & logs
    def clearGPUMemory(self):
        self._check(self._lib.sgdlm_clear_memory(self._h))

    def clearSimulationMemory(self):
        self._check(self._lib.sgdlm_clear_sim_memory(self._h))

    def getLogLevel(self) -> int:
        v = C.c_int()
        self._lib.sgdlm_get_log_level(self._h, C.byref(v))
        return int(v.value)

    def setLogLevel(self, level: int):
        self._lib.sgdlm_set_log_level(self._h, int(level))

    # --------------------------------------------- engine options (GB300)
    def setPrecision(self, precision: str):
        code = {"fp64": L.PRECISION_FP64, "mixed": L.PRECISION_MIXED}[precision]
        self._check(self._lib.sgdlm_set_precision(self._h, code))

    def getPrecision(self) -> str:
        v = C.c_int()
        self._lib.sgdlm_get_precision(self._h, C.byref(v))
        return "fp64" if v.value == L.PRECISION_FP64 else "mixed"

    def setCompat(self, flags: int):
        self._lib.sgdlm_set_compat(self._h, int(flags))

    def setEliminationLevels(self, levels: int):
        """Sparse pre-elimination levels before the dense LU (0 = dense LU only)."""
        self._check(self._lib.sgdlm_set_elimination_levels(self._h, int(levels)))

    def getEliminationInfo(self):
        lv, core = C.c_int(), C.c_int()
        self._lib.sgdlm_get_elimination_info(self._h, C.byref(lv), C.byref(core))
        return {"levels": int(lv.value), "core_n": int(core.value)}

    def setRngState(self, seed: int, epoch: int = 0):
        self._check(self._lib.sgdlm_set_rng_state(self._h, int(seed), int(epoch)))

    def getRngState(self):
        s, e = C.c_uint64(), C.c_uint64()
        self._lib.sgdlm_get_rng_state(self._h, C.byref(s), C.byref(e))
        return int(s.value), int(e.value)

    def getStats(self) -> dict:
        st = L.Stats()
        self._lib.sgdlm_get_stats(self._h, C.byref(st))
        return st.as_dict()

    def getDraws(self):
        """Current draws in the reference's draw-major layouts plus per-draw log|det|."""
        m, P, n = self.m, self.max_p, self.nsim
        lam = np.zeros((m, n), order="F"); th = np.zeros((P, m, n), order="F"); ld = np.zeros(n)
        if not self._check(self._lib.sgdlm_get_draws(self._h, _pd(lam), _pd(th), _pd(ld))):
            return None
        return {"lambdas": lam, "thetas": th, "log_dets": ld}

    # ------------------------------------------------ learned importance proposal
    def setProposal(self, mode: str = "plain", train_steps: int = 500, iters_per_step: int = 4,
                    batch: int = 4096, lr: float = 1e-3, ess_fraction: float = 0.5,
                    seed: int = 20261204):
        """The importance proposal of computeVBPosterior: "plain" (the reference's
        decoupled naive posterior) or "learned" (include/sgdlm.h)."""
        cfg = L.ProposalConfig(L.PROPOSAL_LEARNED if mode == "learned" else L.PROPOSAL_PLAIN,
                               int(train_steps), int(iters_per_step), int(batch), float(lr),
                               float(ess_fraction), int(seed))
        self._check(self._lib.sgdlm_set_proposal(self._h, C.byref(cfg)))

    def getProposal(self) -> dict:
        cfg = L.ProposalConfig()
        self._lib.sgdlm_get_proposal(self._h, C.byref(cfg))
        d = cfg.as_dict()
        d["mode"] = "learned" if d["mode"] == L.PROPOSAL_LEARNED else "plain"
        return d

    def getProposalInfo(self) -> dict:
        info = L.ProposalInfo()
        self._lib.sgdlm_get_proposal_info(self._h, C.byref(info))
        return info.as_dict()

    def proposalSizes(self):
        n, f, o = C.c_size_t(), C.c_int(), C.c_int()
        if not self._check(self._lib.sgdlm_proposal_sizes(self._h, C.byref(n), C.byref(f), C.byref(o))):
            return None
        return int(n.value), int(f.value), int(o.value)

    def getProposalParams(self) -> np.ndarray:
        n, _, _ = self.proposalSizes()
        w = np.zeros(n, dtype=np.float32)
        if not self._check(self._lib.sgdlm_proposal_get_params(self._h, w.ctypes.data)):
            return None
        return w

    def setProposalParams(self, w):
        w = np.ascontiguousarray(w, dtype=np.float32)
        self._check(self._lib.sgdlm_proposal_set_params(self._h, w.ctypes.data))

    def proposalLossAndGradient(self, X, Y, mask):
        """Masked MSE and its gradient (flat parameter layout) on a batch of
        normalised features X (B x F), targets Y and mask (B x O)."""
        X = np.ascontiguousarray(X, dtype=np.float32)
        Y = np.ascontiguousarray(Y, dtype=np.float32)
        M = np.ascontiguousarray(mask, dtype=np.float32)
        n, _, _ = self.proposalSizes()
        g = np.zeros(n, dtype=np.float32)
        loss = C.c_double()
        if not self._check(self._lib.sgdlm_proposal_loss_and_gradient(
                self._h, X.shape[0], X.ctypes.data, Y.ctypes.data, M.ctypes.data, C.byref(loss),
                g.ctypes.data)):
            return None
        return float(loss.value), g

    def getProposalState(self):
        """The last learned call's proposal (m, C, n, s) and the draws' log weights."""
        m, P, n = self.m, self.max_p, self.nsim
        mq = np.zeros((P, m), order="F"); Cq = np.zeros((P, P, m), order="F")
        nq = np.zeros(m); sq = np.zeros(m); lw = np.zeros(n)
        if not self._check(self._lib.sgdlm_get_proposal_state(self._h, _pd(mq), _pd(Cq), _pd(nq),
                                                              _pd(sq), _pd(lw))):
            return None
        return {"m": mq, "C": Cq, "n": nq, "s": sq, "log_weights": lw}

    # ------------------------------------------------------------ LU tuning
    def setLuOptions(self, allow_tensor_cores: bool = True, max_ctas: int = 0):
        self._check(self._lib.sgdlm_set_lu_options(self._h, 1 if allow_tensor_cores else 0,
                                                   int(max_ctas)))

    def setForecastSolver(self, iterative: bool = True):
        self._check(self._lib.sgdlm_set_forecast_solver(self._h, 1 if iterative else 0))

    def setWarpLu(self, enable: bool = True):
        """m <= 32: one warp per draw with partial pivoting (default), or the
        block LU kernels (include/sgdlm.h, sgdlm_set_warp_lu)."""
        self._check(self._lib.sgdlm_set_warp_lu(self._h, 1 if enable else 0))

    def getWarpLu(self):
        en, use = C.c_int(), C.c_int()
        self._lib.sgdlm_get_warp_lu(self._h, C.byref(en), C.byref(use))
        return {"enabled": bool(en.value), "in_use": bool(use.value)}

    def getLuOptions(self):
        tc, mx = C.c_int(), C.c_int()
        self._lib.sgdlm_get_lu_options(self._h, C.byref(tc), C.byref(mx))
        return {"allow_tensor_cores": bool(tc.value), "max_ctas": int(mx.value)}

    def tuneLu(self):
        """Times the batched LU over elimination levels and the tensor-core switch
        and keeps the fastest (include/sgdlm.h, sgdlm_tune_lu)."""
        t = L.LuTuning()
        if not self._check(self._lib.sgdlm_tune_lu(self._h, C.byref(t))):
            return None
        return t.as_dict()

    def launchCount(self) -> int:
        v = C.c_uint64()
        self._lib.sgdlm_get_launch_count(self._h, C.byref(v))
        return int(v.value)

    def stream(self) -> int:
        v = C.c_void_p()
        self._lib.sgdlm_get_stream(self._h, C.byref(v))
        return int(v.value or 0)

    def synchronize(self):
        self._check(self._lib.sgdlm_synchronize(self._h))

    def filterStepDevice(self, d_y: int, d_F: int, d_x: Optional[int], ess_threshold: float,
                         d_forecast: Optional[int] = None, d_weights: Optional[int] = None,
                         d_stats: Optional[int] = None) -> bool:
        """Fused device-resident time step (device pointers as integers); asynchronous."""
        return self._check(self._lib.sgdlm_filter_step_device(
            self._h, C.c_void_p(d_y), C.c_void_p(d_F), C.c_void_p(d_x) if d_x else None,
            float(ess_threshold), C.c_void_p(d_forecast) if d_forecast else None,
            C.c_void_p(d_weights) if d_weights else None, C.c_void_p(d_stats) if d_stats else None))


class Batch:
    """Several engines advanced together: one CUDA-graph launch per time step
    whose branches (one fused step per engine) run concurrently
    (include/sgdlm.h, sgdlm_batch_*).  The engines stay owned by the caller."""

    def __init__(self, engines):
        self._lib = L.lib()
        self.engines = list(engines)
        hs = (L._H * len(self.engines))(*[e._h for e in self.engines])
        self._b = C.c_void_p()
        st = self._lib.sgdlm_batch_create(hs, len(self.engines), C.byref(self._b))
        if st != L.OK:
            raise SGDLMError(f"sgdlm_batch_create failed: {L.STATUS.get(st, st)}")

    def close(self):
        if self._b:
            self._lib.sgdlm_batch_destroy(self._b)
            self._b = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def _ptrs(values):
        if values is None:
            return None
        return (C.c_void_p * len(values))(*[C.c_void_p(v) if v else None for v in values])

    def record(self, d_y, d_F, d_x=None, ess_threshold=0.0, d_forecast=None, d_weights=None,
               d_stats=None):
        """Records one fused step per engine (device pointers as integers, one per engine)."""
        st = self._lib.sgdlm_batch_record(self._b, self._ptrs(d_y), self._ptrs(d_F),
                                          self._ptrs(d_x), float(ess_threshold),
                                          self._ptrs(d_forecast), self._ptrs(d_weights),
                                          self._ptrs(d_stats))
        if st != L.OK:
            raise SGDLMError(f"sgdlm_batch_record failed: {L.STATUS.get(st, st)}")

    def step(self):
        st = self._lib.sgdlm_batch_step(self._b)
        if st != L.OK:
            raise SGDLMError(f"sgdlm_batch_step failed: {L.STATUS.get(st, st)}")

    def autotune(self, replays: int = 3) -> dict:
        t = L.BatchTuning()
        st = self._lib.sgdlm_batch_autotune(self._b, int(replays), C.byref(t))
        if st != L.OK:
            raise SGDLMError(f"sgdlm_batch_autotune failed: {L.STATUS.get(st, st)}")
        return t.as_dict()
