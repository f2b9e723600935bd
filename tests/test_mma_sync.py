"""Host model of the tensor-core LU's bounded MMA waits (no GPU).

The kernel's wait rules (gpusgdlm_gb300/csrc/mma_sync.hpp) are run against a
model of the completion barrier (tests/mma_sync_check.cpp): tiles whose MMAs
complete late or never must never hand out results of an unfinished MMA, every
draw of a CTA that gave its barrier up is marked bad (the pivoting pass redoes
it), and such a CTA issues no further MMAs.  The model also runs the rule
without the drain (flip the phase on a timeout), and shows it hands out
unfinished results in the same scenario.
"""
import ctypes as C
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
DONE, DRAINED, LOST, SKIPPED = 0, 1, 2, 3


@pytest.fixture(scope="module")
def model(tmp_path_factory):
    out = tmp_path_factory.mktemp("mma") / "libmma_model.so"
    r = subprocess.run(["g++", "-O1", "-std=c++17", "-shared", "-fPIC",
                        str(ROOT / "tests" / "mma_sync_check.cpp"), "-o", str(out)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    L = C.CDLL(str(out))
    L.mma_model_run.restype = C.c_int
    L.mma_model_run.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_long, C.c_long,
                                C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
    return L


def run(L, delay, jitter, first=10, drain=100, legacy=False):
    delay = np.asarray(delay, dtype=np.int64)
    jitter = np.asarray(jitter, dtype=np.int64)
    tiles, nt = len(delay), len(jitter)
    status = np.zeros((tiles, nt), dtype=np.int32)
    issued = np.zeros(tiles, dtype=np.int32)
    bad = np.zeros((tiles, nt), dtype=np.int32)
    v = L.mma_model_run(tiles, delay.ctypes.data, nt, jitter.ctypes.data, first, drain,
                        int(legacy), status.ctypes.data, issued.ctypes.data, bad.ctypes.data)
    return v, status, issued, bad


JITTER = [0, 1, 3, 7, 2, 5, 4, 6]


def test_prompt_completions_are_used(model):
    v, status, issued, bad = run(model, [2, 0, 5, 1, 3], JITTER)
    assert v == 0
    assert (status == DONE).all() and not bad.any() and issued.all()


def test_late_completion_is_drained_and_phase_stays_in_step(model):
    # tile 1 completes after the first bound but within the drain
    v, status, issued, bad = run(model, [2, 40, 1, 1, 2], JITTER)
    assert v == 0
    assert (status[1] == DRAINED).all() and bad[1].all()
    # the following tiles wait for their own commits and use them
    assert (status[2:] == DONE).all() and not bad[2:].any() and issued.all()


def test_completion_never_seen_gives_the_barrier_up(model):
    # tile 1 never completes within first + drain (it completes later, out of sight)
    v, status, issued, bad = run(model, [2, 500, 1, 1, 2, 0], JITTER)
    assert v == 0
    assert (status[1] == LOST).all() and bad[1].all()
    assert not issued[2:].any()              # no MMAs after the CTA gave up
    assert (status[2:] == SKIPPED).all()     # and no more waits
    assert bad[2:].all()                     # every later draw goes to the pivoting pass


def test_some_threads_see_the_late_completion(model):
    # the completion lands while some threads are still in their drain window and
    # others have given up: nobody uses an unfinished tile, and the CTA gives up
    jit = [0, 0, 0, 0, 60, 60, 60, 60]
    v, status, issued, bad = run(model, [1, 150, 1, 1], jit, first=10, drain=100)
    assert v == 0
    assert set(status[1]) == {LOST, DRAINED}
    assert not issued[2:].any() and bad[2:].all()


def test_flip_on_timeout_rule_hands_out_unfinished_tiles(model):
    # without the drain the late completion of tile 1 satisfies tile 2's wait
    v, status, issued, bad = run(model, [2, 40, 200, 1], JITTER, legacy=True)
    assert v > 0
