"""ctypes binding of the C ABI in include/sgdlm.h.

The CUDA library is in-tree (gpusgdlm_gb300/libsgdlm_gb300.so, built by
gpusgdlm_gb300/build.py).  There is no fallback: if the library is missing or
does not load, importing the engine raises.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

HERE = Path(__file__).resolve().parent
LIB_PATH = Path(os.environ.get("SGDLM_GB300_LIB", HERE / "libsgdlm_gb300.so"))

OK = 0
STATUS = {
    0: "SGDLM_OK",
    1: "SGDLM_ERR_BAD_DIM",
    2: "SGDLM_ERR_NOT_INIT",
    3: "SGDLM_ERR_WRONG_STATE",
    4: "SGDLM_ERR_SIM_NOT_INIT",
    5: "SGDLM_ERR_DEVICE",
    6: "SGDLM_ERR_BAD_ARG",
    7: "SGDLM_ERR_NO_DEVICE",
    8: "SGDLM_ERR_OUT_OF_MEMORY",
    9: "SGDLM_ERR_UNSUPPORTED",
    10: "SGDLM_ERR_EVO_DISABLED",
}
PRECISION_FP64 = 0
PRECISION_MIXED = 1
COMPAT_UNSCALED_EVOLUTION = 1
COMPAT_BETA_NO_BOOST = 2
COMPAT_REFERENCE = 3
COMPAT_NONE = 0


class Stats(C.Structure):
    _fields_ = [
        ("ess", C.c_double),
        ("sum_det_weights", C.c_double),
        ("max_log_det", C.c_double),
        ("draws_pivoted", C.c_uint64),
        ("draws_singular", C.c_uint64),
        ("gamma_cap_hits", C.c_uint64),
        ("newton_fallbacks", C.c_uint64),
        ("ms_sample", C.c_double),
        ("ms_lu", C.c_double),
        ("ms_weights", C.c_double),
        ("ms_vb", C.c_double),
        ("ms_total", C.c_double),
        ("ms_lu_forecast", C.c_double),
        ("forecast_draws_factored", C.c_uint64),
        ("draws_pivoted_full", C.c_uint64),
    ]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class ProposalConfig(C.Structure):
    _fields_ = [
        ("mode", C.c_int),
        ("train_steps", C.c_int),
        ("iters_per_step", C.c_int),
        ("batch", C.c_int),
        ("lr", C.c_double),
        ("ess_fraction", C.c_double),
        ("seed", C.c_uint64),
    ]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class ProposalInfo(C.Structure):
    _fields_ = [
        ("training_calls", C.c_uint64),
        ("samples", C.c_uint64),
        ("adam_steps", C.c_uint64),
        ("learned_calls", C.c_uint64),
        ("fallbacks", C.c_uint64),
        ("last_loss", C.c_double),
        ("ess_learned", C.c_double),
        ("ess_plain", C.c_double),
        ("deployed", C.c_int),
        ("used_learned", C.c_int),
    ]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class LuTuning(C.Structure):
    _fields_ = [
        ("levels", C.c_int),
        ("tensor_cores", C.c_int),
        ("core_n", C.c_int),
        ("ms", C.c_double),
        ("ms_candidates", C.c_double * 8),
    ]

    def as_dict(self):
        d = {f: getattr(self, f) for f, _ in self._fields_}
        d["ms_candidates"] = list(self.ms_candidates)
        return d


class BatchTuning(C.Structure):
    _fields_ = [
        ("buckets", C.c_int),
        ("lu_plans_kept", C.c_int),
        ("concurrency", C.c_int),
        ("ms_untuned", C.c_double),
        ("ms_per_step", C.c_double),
        ("ms_candidates", C.c_double * 4),
    ]

    def as_dict(self):
        d = {f: getattr(self, f) for f, _ in self._fields_}
        d["ms_candidates"] = list(self.ms_candidates)
        return d


PROPOSAL_PLAIN = 0
PROPOSAL_LEARNED = 1

_H = C.c_void_p
_sz, _i, _u, _u64, _d = C.c_size_t, C.c_int, C.c_uint, C.c_uint64, C.c_double
_Pd, _Pu, _Psz, _Pi, _Pu64 = (C.POINTER(C.c_double), C.POINTER(C.c_uint), C.POINTER(C.c_size_t),
                              C.POINTER(C.c_int), C.POINTER(C.c_uint64))

SIGNATURES = {
    "sgdlm_create": [_sz, C.POINTER(_H)],
    "sgdlm_destroy": [_H],
    "sgdlm_init_memory": [_H, _sz, _sz],
    "sgdlm_clear_memory": [_H],
    "sgdlm_get_no_series": [_H, _Psz],
    "sgdlm_get_max_p": [_H, _Psz],
    "sgdlm_get_no_gpus": [_H, _Psz],
    "sgdlm_init_sim_memory": [_H, _sz, _sz],
    "sgdlm_clear_sim_memory": [_H],
    "sgdlm_get_nsim": [_H, _Psz],
    "sgdlm_get_nsim_batch": [_H, _Psz],
    "sgdlm_is_prior": [_H, _Pi],
    "sgdlm_set_is_prior": [_H, _i],
    "sgdlm_get_parameters": [_H, _Pd, _Pd, _Pd, _Pd],
    "sgdlm_set_parameters": [_H, _Pd, _Pd, _Pd, _Pd],
    "sgdlm_get_discount_factors": [_H, _Pd, _Pd],
    "sgdlm_set_discount_factors": [_H, _Pd, _Pd],
    "sgdlm_get_parental_sets": [_H, _Pu, _Pu],
    "sgdlm_set_parental_sets": [_H, _Pu, _Pu],
    "sgdlm_compute_posterior": [_H, _Pd, _Pd],
    "sgdlm_compute_vb_posterior": [_H, _Pd, _Pd, _Pd, _Pd, _Pd, _Pd],
    "sgdlm_compute_prior": [_H, _i],
    "sgdlm_init_forecast_priors": [_H],
    "sgdlm_evolve_forecast_samples": [_H],
    "sgdlm_get_evolution_matrix_configuration": [_H, _Pi],
    "sgdlm_manage_evo_memory": [_H, _i],
    "sgdlm_get_evolution_matrix": [_H, _Pd],
    "sgdlm_set_evolution_matrix": [_H, _Pd],
    "sgdlm_compute_evo_prior": [_H, _Pd, _i],
    "sgdlm_evolve_forecast_samples_evo": [_H, _Pd],
    "sgdlm_compute_forecast": [_H, _Pd, _Pd, _Pd, _Pd, _i],
    "sgdlm_get_draws": [_H, _Pd, _Pd, _Pd],
    "sgdlm_set_precision": [_H, _i],
    "sgdlm_get_precision": [_H, _Pi],
    "sgdlm_set_compat": [_H, _u],
    "sgdlm_set_elimination_levels": [_H, _i],
    "sgdlm_get_elimination_info": [_H, _Pi, _Pi],
    "sgdlm_get_compat": [_H, C.POINTER(C.c_uint)],
    "sgdlm_set_rng_state": [_H, _u64, _u64],
    "sgdlm_get_rng_state": [_H, _Pu64, _Pu64],
    "sgdlm_get_stats": [_H, C.POINTER(Stats)],
    "sgdlm_set_log_level": [_H, _i],
    "sgdlm_get_log_level": [_H, _Pi],
    "sgdlm_last_error": [_H],
    "sgdlm_set_proposal": [_H, C.POINTER(ProposalConfig)],
    "sgdlm_get_proposal": [_H, C.POINTER(ProposalConfig)],
    "sgdlm_get_proposal_info": [_H, C.POINTER(ProposalInfo)],
    "sgdlm_proposal_sizes": [_H, _Psz, _Pi, _Pi],
    "sgdlm_proposal_get_params": [_H, C.c_void_p],
    "sgdlm_proposal_set_params": [_H, C.c_void_p],
    "sgdlm_proposal_loss_and_gradient": [_H, _sz, C.c_void_p, C.c_void_p, C.c_void_p, _Pd,
                                         C.c_void_p],
    "sgdlm_get_proposal_state": [_H, _Pd, _Pd, _Pd, _Pd, _Pd],
    "sgdlm_filter_step_device": [_H, C.c_void_p, C.c_void_p, C.c_void_p, _d, C.c_void_p,
                                 C.c_void_p, C.c_void_p],
    "sgdlm_set_lu_options": [_H, _i, _i],
    "sgdlm_get_lu_options": [_H, _Pi, _Pi],
    "sgdlm_set_forecast_solver": [_H, _i],
    "sgdlm_set_warp_lu": [_H, _i],
    "sgdlm_get_warp_lu": [_H, C.POINTER(_i), C.POINTER(_i)],
    "sgdlm_tune_lu": [_H, C.POINTER(LuTuning)],
    "sgdlm_batch_create": [C.POINTER(_H), _sz, C.POINTER(C.c_void_p)],
    "sgdlm_batch_destroy": [C.c_void_p],
    "sgdlm_batch_record": [C.c_void_p, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p),
                           C.POINTER(C.c_void_p), _d, C.POINTER(C.c_void_p),
                           C.POINTER(C.c_void_p), C.POINTER(C.c_void_p)],
    "sgdlm_batch_step": [C.c_void_p],
    "sgdlm_batch_autotune": [C.c_void_p, _i, C.POINTER(BatchTuning)],
    "sgdlm_get_stream": [_H, C.POINTER(C.c_void_p)],
    "sgdlm_synchronize": [_H],
    "sgdlm_get_launch_count": [_H, _Pu64],
    "sgdlm_log_det_noalloc": [_sz, _sz, _sz, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                              C.c_void_p],
}

_lib = None


def lib() -> C.CDLL:
    """Loads the CUDA library (raises if it is absent: there is no CPU path)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise ImportError(
                f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`"
            )
        L = C.CDLL(str(LIB_PATH))
        for name, args in SIGNATURES.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = C.c_char_p if name == "sgdlm_last_error" else C.c_int
        _lib = L
    return _lib
