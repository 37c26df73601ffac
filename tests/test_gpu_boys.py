"""The device Boys functions, evaluated on the GPU by the code the kernels run
(fock_boys_eval), against mpmath (tests/golden/boys_mpmath.json, 40 digits)
and against the oracle's restatement of the reference's LUT function
(boys/src/lib.rs:58-81 with the stored boys/src/lut.rs table), including the
index clamp in [29.85, 30) and the asymptotic branch from t = 30."""
import ctypes as C

import numpy as np
import pytest

from fock_gb300 import _lib as L

pytestmark = pytest.mark.gpu

FP64_REL = 1e-14   # FP64 Taylor table + downward recursion (ERI kernels), every order 0..12
MD_REL = 1e-14     # runtime-order form of the one-electron / MD kernels
FP32_REL = 5e-6    # FP32 form of the mixed-precision kernels (4 Taylor terms, float recursion)


def _eval(lib, form, order, T):
    T = np.ascontiguousarray(T, dtype=np.float64)
    out = np.zeros((len(T), order + 1))
    rc = lib.fock_boys_eval(0, form, order, T.ctypes.data_as(C.POINTER(C.c_double)), len(T),
                            out.ctypes.data_as(C.POINTER(C.c_double)))
    assert rc == 0, rc
    return out


@pytest.mark.parametrize("form,tol", [(L.FOCK_BOYS_FP64, FP64_REL), (L.FOCK_BOYS_MD, MD_REL),
                                      (L.FOCK_BOYS_FP32, FP32_REL)])
def test_device_boys_vs_mpmath(gpu_lib, golden_boys, form, tol):
    rows = np.array(golden_boys["rows"])
    T, ref = rows[:, 0], rows[:, 1:]
    worst = 0.0
    for order in range(golden_boys["orders"]):
        got = _eval(gpu_lib, form, order, T)
        rel = np.abs(got - ref[:, :order + 1]) / np.abs(ref[:, :order + 1])
        if form == L.FOCK_BOYS_FP32:
            # FP32 values below the float range are flushed; compare where representable
            rel = rel[ref[:, :order + 1] > 1e-30]
        worst = max(worst, float(rel.max()))
    assert worst < tol, (form, worst)


def test_device_reference_boys_matches_oracle(gpu_lib, oracle_lib):
    # dense near the LUT nodes, across the [29.85, 30) clamp and the t = 30 switch
    T = np.concatenate([np.linspace(0.0, 29.8, 600), np.linspace(29.8, 30.2, 401), [0.0, 1e-17, 0.15 * 199],
                        np.linspace(30.0, 60.0, 31)])
    T = np.abs(T)
    got = _eval(gpu_lib, L.FOCK_BOYS_REFERENCE, 10, T)
    worst = 0.0
    for i, t in enumerate(T):
        for n in range(11):
            ref = oracle_lib.boys(t, n, oracle_lib.BOYS_LUT)
            worst = max(worst, abs(got[i, n] - ref) / abs(ref))
    assert worst < 1e-13, worst
    # the clamp: in [29.85, 30) the reference interpolates towards entry 199 (not 200),
    # which the exact function does not do: the device must show the same defect
    t = 29.9
    dev = _eval(gpu_lib, L.FOCK_BOYS_REFERENCE, 0, [t])[0, 0]
    exact = oracle_lib.boys(t, 0, oracle_lib.EXACT)
    assert abs(dev - exact) / exact > 1e-3


def test_boys_eval_rejects_bad_input(gpu_lib):
    out = np.zeros(4)
    T = np.array([1.0, -1.0])
    dp = C.POINTER(C.c_double)
    assert gpu_lib.fock_boys_eval(0, L.FOCK_BOYS_FP64, 2, T.ctypes.data_as(dp), 2, out.ctypes.data_as(dp)) == -1
    T = np.array([1.0])
    assert gpu_lib.fock_boys_eval(0, L.FOCK_BOYS_REFERENCE, 11, T.ctypes.data_as(dp), 1, out.ctypes.data_as(dp)) == -1
    assert gpu_lib.fock_boys_eval(0, 7, 1, T.ctypes.data_as(dp), 1, out.ctypes.data_as(dp)) == -1
