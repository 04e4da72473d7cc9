"""ctypes view of oracle/liboracle.so -- the CPU restatement used as the parity
reference in tests/ and as the timed CPU baseline ("port") of bench.py.

Test infrastructure only; the product library never imports this module.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None
KIND_FULL, KIND_NUMBER, KIND_SZ = 0, 1, 2


def build():
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "liboracle.so")
        if not os.path.exists(path):
            build()
        L = ctypes.CDLL(path)
        P = ctypes.c_void_p
        dp = ctypes.POINTER(ctypes.c_double)
        ip = ctypes.POINTER(ctypes.c_int)
        L.or_create.restype = P
        L.or_create.argtypes = [ctypes.c_int] * 6
        L.or_destroy.argtypes = [P]
        L.or_dim.restype = ctypes.c_int64
        L.or_dim.argtypes = [P]
        L.or_states.argtypes = [P, ctypes.POINTER(ctypes.c_uint32)]
        L.or_set_initial.argtypes = [P, ctypes.c_int, ip, dp, dp]
        L.or_set_ops.argtypes = [P, ctypes.c_int, ip, ip, dp, ctypes.c_int]
        L.or_set_ham_triplets.argtypes = [P, ctypes.c_int, ip, ip, dp]
        L.or_set_ham_integrals.argtypes = [P, dp, dp, ctypes.c_int]
        L.or_ham_nnz.restype = ctypes.c_int64
        L.or_ham_nnz.argtypes = [P]
        L.or_ham_nops.argtypes = [P]
        L.or_ham_csr.argtypes = [P, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int32), dp]
        L.or_apply_h.argtypes = [P, dp, dp]
        L.or_apply_h_rows.argtypes = [P, dp, ctypes.POINTER(ctypes.c_int64), ctypes.c_int, dp]
        L.or_evolve.argtypes = [P, dp, dp]
        L.or_energy_gradient.argtypes = [P, dp, dp, dp]
        L.or_gradient_comp.argtypes = [P, dp, dp, dp]
        L.or_hessian_comp.argtypes = [P, dp, dp]
        L.or_gradient_proj.argtypes = [P, dp, dp, dp, dp]
        L.or_hessian_ops.argtypes = [P, dp, dp]
        L.or_exc_apply.argtypes = [ctypes.c_uint32] + [ctypes.c_int] * 4 + [ctypes.POINTER(ctypes.c_uint32), ip]
        L.or_basis_size.restype = ctypes.c_int64
        L.or_basis_size.argtypes = [ctypes.c_int] * 5
        L.or_num_threads.restype = ctypes.c_int
        _LIB = L
    return _LIB


def _d(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _i(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


def exc_apply(state, e):
    """(kind, partner, sign) of the reference rule for one 0-based excitation."""
    p = ctypes.c_uint32()
    s = ctypes.c_int()
    k = lib().or_exc_apply(int(state), int(e[0]), int(e[1]), int(e[2]), int(e[3]), ctypes.byref(p), ctypes.byref(s))
    return k, p.value, s.value


class Oracle:
    """One problem: sector basis, excitations, Hamiltonian, initial state."""

    def __init__(self, nq, kind, ne, na, nb, cplx=False):
        self.L = lib()
        self.h = self.L.or_create(nq, kind, ne, na, nb, int(cplx))
        self.nq, self.cplx = nq, cplx
        self.D = self.L.or_dim(self.h)
        self.nparams = 0
        self.nops = 0

    def __del__(self):
        if getattr(self, "h", None):
            self.L.or_destroy(self.h)
            self.h = None

    def states(self):
        out = np.zeros(self.D, dtype=np.uint32)
        self.L.or_states(self.h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)))
        return out

    def set_initial(self, idx, re, im=None):
        idx = np.ascontiguousarray(idx, dtype=np.int32)
        re = np.ascontiguousarray(re, dtype=np.float64)
        im = np.zeros_like(re) if im is None else np.ascontiguousarray(im, dtype=np.float64)
        assert self.L.or_set_initial(self.h, len(idx), _i(idx), _d(re), _d(im)) == 0

    def set_ops(self, ops0, param0, scale):
        """ops0: (n,4) 0-based with -1 absent; param0: 0-based parameter of each op."""
        ops0 = np.ascontiguousarray(ops0, dtype=np.int32).reshape(-1, 4)
        param0 = np.ascontiguousarray(param0, dtype=np.int32)
        scale = np.ascontiguousarray(scale, dtype=np.float64)
        self.nops = len(ops0)
        self.nparams = int(param0.max()) + 1
        self.L.or_set_ops(self.h, self.nops, _i(ops0), _i(param0), _d(scale), self.nparams)

    def set_ham_triplets(self, i0, j0, v):
        i0 = np.ascontiguousarray(i0, dtype=np.int32)
        j0 = np.ascontiguousarray(j0, dtype=np.int32)
        v = np.ascontiguousarray(v, dtype=np.float64)
        self.L.or_set_ham_triplets(self.h, len(v), _i(i0), _i(j0), _d(v))

    def set_ham_integrals(self, h1, g2, csr=True):
        h1 = np.ascontiguousarray(h1, dtype=np.float64)
        g2 = np.ascontiguousarray(g2, dtype=np.float64)
        self.L.or_set_ham_integrals(self.h, _d(h1), _d(g2), 1 if csr else 2)

    def csr(self):
        nnz = self.L.or_ham_nnz(self.h)
        rp = np.zeros(self.D + 1, dtype=np.int64)
        col = np.zeros(nnz, dtype=np.int32)
        val = np.zeros(nnz, dtype=np.float64)
        self.L.or_ham_csr(self.h, rp.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                          col.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), _d(val))
        return rp, col, val

    def _w(self):
        return 2 if self.cplx else 1

    def apply_h(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.zeros_like(x)
        assert self.L.or_apply_h(self.h, _d(x), _d(y)) == 0
        return y

    def apply_h_rows(self, x, rows):
        x = np.ascontiguousarray(x, dtype=np.float64)
        rows = np.ascontiguousarray(rows, dtype=np.int64)
        y = np.zeros(len(rows) * self._w())
        assert self.L.or_apply_h_rows(self.h, _d(x), rows.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), len(rows), _d(y)) == 0
        return y

    def evolve_ops(self, ang_ops):
        a = np.ascontiguousarray(ang_ops, dtype=np.float64)
        out = np.zeros(self.D * self._w())
        self.L.or_evolve(self.h, _d(a), _d(out))
        return out

    def energy_gradient_ops(self, ang_ops):
        a = np.ascontiguousarray(ang_ops, dtype=np.float64)
        E = np.zeros(1)
        g = np.zeros(self.nops)
        self.L.or_energy_gradient(self.h, _d(a), _d(E), _d(g))
        return E[0], g

    def gradient_proj_ops(self, ang_ops, proj):
        """(<proj|psi>, d<proj|psi>/dtheta_op): the projected sweep (evolveDerivativeProj)."""
        a = np.ascontiguousarray(ang_ops, dtype=np.float64)
        pr = np.ascontiguousarray(proj, dtype=np.float64)
        assert pr.size == self.D * self._w()
        ov = np.zeros(1)
        g = np.zeros(self.nops)
        self.L.or_gradient_proj(self.h, _d(a), _d(pr), _d(ov), _d(g))
        return ov[0], g

    def gradient_comp(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        E = np.zeros(1)
        g = np.zeros(self.nparams)
        self.L.or_gradient_comp(self.h, _d(x), _d(E), _d(g))
        return E[0], g

    def hessian_comp(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        H = np.zeros((self.nparams, self.nparams))
        self.L.or_hessian_comp(self.h, _d(x), _d(H))
        return H
