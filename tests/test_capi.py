"""C-ABI checks that need no GPU: the library loads, exports every entry point
declared in include/sgdlm.h, and fails cleanly without a device or a handle."""
import ctypes as C
import re
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]


def declared_symbols():
    text = (ROOT / "include" / "sgdlm.h").read_text()
    return sorted(set(re.findall(r"\b(sgdlm_[a-z_0-9]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(built_lib):
    lib = C.CDLL(str(built_lib))
    names = declared_symbols()
    assert len(names) >= 40
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_the_header(built_lib):
    from gpusgdlm_gb300 import _lib

    assert set(declared_symbols()) == set(_lib.SIGNATURES)


def test_null_handle_is_rejected(built_lib):
    from gpusgdlm_gb300 import _lib

    L = _lib.lib()
    assert L.sgdlm_init_memory(None, 4, 2) == 6
    assert L.sgdlm_compute_prior(None, 0) == 6
    assert L.sgdlm_destroy(None) == 0
    assert L.sgdlm_create(1, None) == 6


def test_sp_encoding_matches_r_na():
    from gpusgdlm_gb300 import NA_UNSIGNED, encode_sp

    sp = np.array([[np.nan, 5.0], [-1, 3.0], [None, 99]], dtype=object)
    out = encode_sp(sp, m=4)
    assert out.dtype == np.uint32 and out.flags.f_contiguous
    assert out[0, 0] == NA_UNSIGNED and out[1, 0] == NA_UNSIGNED and out[2, 0] == NA_UNSIGNED
    assert out[0, 1] == 5 and out[1, 1] == 3
    assert out[2, 1] == NA_UNSIGNED  # >= m*m marks an external predictor
    assert NA_UNSIGNED == 2147483648
