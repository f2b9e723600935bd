"""The reference-interface adapter (libsgdlm_hostwrapper.so): the reference's
C++ engine interface SGDLM::HostWrapper<double> and its factory
(rSGDLM/src/SGDLM/HostWrapper.hpp:13-99, HostWrapperFactory.hpp:15-26) on the
GB300 engine.

CPU: the library exports the factory, its vtable layout equals the one a caller
compiled against the reference's own header sees (when the reference checkout is
at hand), the adapter compiles against that header, and construction without a
device gives an inert object (the reference's behaviour with no GPU).
GPU: one filter step through the interface equals the same step through the
C ABI (same default Philox stream), and the evolution-matrix methods round-trip.
"""
import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
PKG = ROOT / "gpusgdlm_gb300"


def reference_src():
    ref = os.environ.get("SGDLM_REFERENCE") or str(ROOT.parent / "reference")
    src = Path(ref) / "rSGDLM" / "src"
    return src if (src / "SGDLM" / "HostWrapper.hpp").exists() else None


def gxx(args):
    r = subprocess.run(["g++", "-std=c++17", *args], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return r


@pytest.fixture(scope="module")
def harness(built_lib, tmp_path_factory):
    out = tmp_path_factory.mktemp("hw") / "libhw_check.so"
    gxx(["-O1", "-fPIC", "-shared", str(ROOT / "tests" / "hostwrapper_check.cpp"),
         "-I", str(ROOT / "include"), "-o", str(out), "-L", str(PKG), "-lsgdlm_hostwrapper",
         f"-Wl,-rpath,{PKG}"])
    L = C.CDLL(str(out))
    L.hw_no_device.restype = C.c_int
    L.hw_filter_step.restype = C.c_int
    return L


def test_factory_symbols_exported(built_lib):
    lib = PKG / "libsgdlm_hostwrapper.so"
    assert lib.exists()
    r = subprocess.run(["nm", "-DC", str(lib)], capture_output=True, text=True)
    forms = [ln for ln in r.stdout.splitlines()
             if " T " in ln and "SGDLM::HostWrapperFactory<double>::create(" in ln]
    assert len(forms) == 3, r.stdout


def test_vtable_layout_matches_reference_header(tmp_path):
    src = reference_src()
    if src is None:
        pytest.skip("the reference checkout is not at hand")
    own, ref = tmp_path / "own", tmp_path / "ref"
    code = str(ROOT / "tests" / "hostwrapper_layout.cpp")
    gxx([code, "-I", str(ROOT / "include"), "-o", str(own)])
    gxx([code, "-DSGDLM_USE_REFERENCE_HEADERS", "-I", str(src), "-o", str(ref)])
    a = subprocess.run([str(own)], capture_output=True, text=True, check=True).stdout
    b = subprocess.run([str(ref)], capture_output=True, text=True, check=True).stdout
    assert a.count("\n") == 28 and a == b


def test_adapter_compiles_against_reference_header():
    src = reference_src()
    if src is None:
        pytest.skip("the reference checkout is not at hand")
    gxx(["-fsyntax-only", "-DSGDLM_USE_REFERENCE_HEADERS", "-I", str(src),
         str(PKG / "csrc" / "host_wrapper.cpp")])


def test_construction_without_device_is_inert(harness):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a device is present")
    assert harness.hw_no_device() == 0


@pytest.mark.gpu
def test_filter_step_through_interface_equals_c_abi(harness):
    from gpusgdlm_gb300 import SGDLM
    from test_gpu_parity import readme_inputs

    d = readme_inputs(100)
    m, P = d["m"], d["P"]
    n = 2000
    spu = np.asfortranarray(np.where(np.isnan(d["sp"]), 2147483648,
                                     np.nan_to_num(d["sp"])).astype(np.uint32))
    p = np.ascontiguousarray(d["p"], dtype=np.uint32)
    a = np.zeros((P, m), order="F")
    R = np.asfortranarray(np.repeat((0.05 * np.eye(P))[:, :, None], m, axis=2))
    r, c = np.full(m, 1.0), np.full(m, 0.01)
    beta, delta = np.ascontiguousarray(d["beta"]), np.asfortranarray(d["Delta"])
    y = np.ascontiguousarray(d["y"][5])
    F = d["predictors"](5, d["y"][5])
    x = d["predictors"](6, None)

    dp = C.POINTER(C.c_double)
    P_ = lambda v: v.ctypes.data_as(dp)  # noqa: E731
    om, oC = np.zeros((P, m), order="F"), np.zeros((P, P, m), order="F")
    on, os_, ow, oy = np.zeros(m), np.zeros(m), np.zeros(n), np.zeros((m, n), order="F")
    osum = C.c_double()
    flags = np.zeros(8, dtype=np.int32)
    st = harness.hw_filter_step(
        C.c_size_t(m), C.c_size_t(P), p.ctypes.data_as(C.c_void_p), spu.ctypes.data_as(C.c_void_p),
        P_(beta), P_(delta), P_(a), P_(R), P_(r), P_(c), P_(y), P_(F), P_(x), C.c_size_t(n),
        P_(om), P_(oC), P_(on), P_(os_), P_(ow), C.byref(osum), P_(oy),
        flags.ctypes.data_as(C.c_void_p))
    assert st == 0
    assert list(flags) == [m, P, 1, 0, 1, n, 0, 1]

    s = SGDLM(1, strict=True)  # default precision and Philox stream, as the factory's
    s.setSimultaneousParents(d["p"], d["sp"])
    s.setDiscountFactors(d["beta"], d["Delta"])
    s.setPriorParameters(a, R, r, c)
    s.computePosterior(y, F)
    vb = s.computeVBPosterior(n, n)
    s.computePrior()
    yf = s.computeForecast(n, n, x)
    np.testing.assert_array_equal(om, vb["m"])
    np.testing.assert_array_equal(oC, vb["C"])
    np.testing.assert_array_equal(on, vb["n"])
    np.testing.assert_array_equal(os_, vb["s"])
    np.testing.assert_array_equal(ow, vb["IS_weights"])
    assert osum.value == vb["sum_det_weights"]
    np.testing.assert_array_equal(oy, yf)


@pytest.mark.gpu
def test_evolution_matrix_entry_points(built_lib):
    from gpusgdlm_gb300 import SGDLM

    m, P = 3, 2
    s = SGDLM(1, strict=False)
    s.setSimultaneousParents([1, 2, 0], np.full((P, m), np.nan))
    assert s.getEvolutionMatrixConfiguration() is False
    G = np.asfortranarray(np.arange(P * P * m, dtype=float).reshape(P, P, m))
    s.setEvolutionMatrix(G)
    assert s.last_status == 10  # SGDLM_ERR_EVO_DISABLED, as HostWrapperImpl.cu:1258-1265
    s.manageEvoMemory(True)
    assert s.getEvolutionMatrixConfiguration() is True
    np.testing.assert_array_equal(s.getEvolutionMatrix(), np.zeros((P, P, m)))
    s.setEvolutionMatrix(G)
    np.testing.assert_array_equal(s.getEvolutionMatrix(), G)
    s.manageEvoMemory(False)
    assert s.getEvolutionMatrixConfiguration() is False
    assert s.getEvolutionMatrix() is None and s.last_status == 10
