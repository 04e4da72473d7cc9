"""Argument checking of the reference-compatible C ABI (AnsatzSynthInterface.cpp):
the same status codes as the reference for null handles, empty inputs and out of
range operators.  These paths return before any GPU work, so they run on CPU."""
import ctypes

import numpy as np

from ansatzevolve_gb300 import lib, dptr, iptr


def test_null_context_codes():
    L = lib()
    a = np.zeros(3)
    i = np.ones(3, dtype=np.int32)
    assert L.cleanup(None) == 1
    assert L.setExcitation(1, iptr(i), iptr(i), None) == 1
    assert L.setHamiltonian(1, iptr(i), iptr(i), dptr(a), None) == 1
    assert L.setInitialState(4, 1, iptr(i), dptr(a), None) == 1
    assert L.getEnergy(1, dptr(a), dptr(a), None) == 1
    assert L.getGradient_COMP(1, dptr(a), dptr(a), None) == 1
    assert L.getHessian_COMP(1, dptr(a), dptr(a), None) == 1
    assert L.getFinalState(1, dptr(a), 4, dptr(a), None) == 1


def test_argument_codes_and_cleanup():
    L = lib()
    ctx = ctypes.c_void_p(L.init())
    assert ctx.value
    a = np.zeros(4)
    i = np.ones(4, dtype=np.int32)
    assert L.setExcitation(0, iptr(i), iptr(i), ctx) == 2
    ops = np.array([200, 1, 0, 0], dtype=np.int32)  # operators[n*j+i], n = 1
    assert L.setExcitation(1, iptr(ops), iptr(i), ctx) == 3
    ops = np.array([1, 2, 0, 0], dtype=np.int32)
    bad_order = np.array([5], dtype=np.int32)
    assert L.setExcitation(1, iptr(ops), iptr(bad_order), ctx) == 5
    assert L.setHamiltonian(0, iptr(i), iptr(i), dptr(a), ctx) == 2
    assert L.setInitialState(4, 0, iptr(i), dptr(a), ctx) == 2
    assert L.setInitialState(0, 1, iptr(i), dptr(a), ctx) == 2
    assert L.getEnergy(1, None, dptr(a), ctx) == 2
    assert L.getEnergy(0, dptr(a), dptr(a), ctx) == 3
    assert L.getFinalState(1, dptr(a), 4, None, ctx) == 3
    assert L.getFinalState(1, dptr(a), 0, dptr(a), ctx) == 4
    assert L.getFinalState(0, dptr(a), 4, dptr(a), ctx) == 5
    assert L.getGradient_COMP(1, dptr(a), None, ctx) == 3
    assert L.getGradient_COMP(0, dptr(a), dptr(a), ctx) == 4
    assert L.getHessian_COMP(1, dptr(a), None, ctx) == 3
    assert L.getHessian_COMP(0, dptr(a), dptr(a), ctx) == 4
    # incomplete setup: evaluation fails with the reference's "computation failed" codes
    assert L.getEnergy(1, dptr(a), dptr(a), ctx) == 3
    assert L.getGradient_COMP(1, dptr(a), dptr(a), ctx) == 5
    assert L.cleanup(ctypes.byref(ctx)) == 0
    assert ctx.value is None
    assert L.cleanup(ctypes.byref(ctx)) == 0


def test_extension_status_codes():
    """The C ABI extensions (per-operator derivatives, batched energies, the optimise /
    properties verbs) follow the same codes: 1 for a null handle, 2 for bad arguments,
    3 when the setup is missing (the first evaluation fails before any GPU work)."""
    L = lib()
    a = np.zeros(4)
    nr = ctypes.c_int()
    assert L.getGradient(4, dptr(a), dptr(a), None) == 1
    assert L.getHessian(4, dptr(a), dptr(a), None) == 1
    assert L.getExpectationValues(1, 4, dptr(a), dptr(a), None) == 1
    assert L.iterativeOptimise(4, dptr(a), dptr(a), None) == 1
    assert L.generatePathsForSubspace(2, dptr(a), ctypes.byref(nr), dptr(a), None) == 1
    assert L.writeProperties(1, 4, dptr(a), 3, None, None) == 1
    assert L.setNumberOfOverlapsToCompute(2, None) == 1
    ctx = ctypes.c_void_p(L.init())
    try:
        assert L.setNumberOfOverlapsToCompute(0, ctx) == 2
        assert L.setNumberOfOverlapsToCompute(3, ctx) == 0
        assert L.getGradient(0, dptr(a), dptr(a), ctx) == 2
        assert L.getHessian(4, None, dptr(a), ctx) == 2
        assert L.getExpectationValues(0, 4, dptr(a), dptr(a), ctx) == 2
        assert L.iterativeOptimise(4, None, dptr(a), ctx) == 2
        assert L.generatePathsForSubspace(0, dptr(a), ctypes.byref(nr), dptr(a), ctx) == 2
        assert L.writeProperties(0, 4, dptr(a), 3, None, ctx) == 2
        assert L.getGradient(4, dptr(a), dptr(a), ctx) == 3
        assert L.getExpectationValues(1, 4, dptr(a), dptr(a), ctx) == 3
        assert L.generatePathsForSubspace(2, dptr(a), ctypes.byref(nr), dptr(a), ctx) == 3
    finally:
        L.cleanup(ctypes.byref(ctx))
