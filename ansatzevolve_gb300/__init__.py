"""GB300-native statevector engine for TUPS / U3 fermionic ansatze.

The product is the in-tree shared library ``libansatzevolve_gb300.so``: hand-written
sm_103a CUDA kernels behind a thin C ABI (``include/aegpu.h``) and, on top of it,
the reference's own drop-in interface -- the C++ ``stateAnsatzManager`` and the
``AnsatzSynthInterface`` C functions (``include/AnsatzSynthInterface.h``).
This module only loads that library with ctypes and mirrors the reference's
Python binding (PyAnsatzEvolve.cpp:17-148) on top of the C ABI.  There is no
CPU implementation of the path here: without the library or a CUDA device every
entry point raises.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libansatzevolve_gb300.so")
_LIB = None

HAM_AUTO, HAM_STORED, HAM_ON_THE_FLY = 0, 1, 2
TUNE_PASS_OPS, TUNE_CTAS_PER_SM, TUNE_OTF_THREADS, TUNE_SPMV_TPR, TUNE_PDL, TUNE_REUSE_HPSI, TUNE_FLIP = 1, 2, 3, 4, 5, 6, 7
TUNE_HALF = 8
BASIS_FULL, BASIS_NUMBER, BASIS_SZ = 0, 1, 2
PROP_HESSIAN, PROP_OVERLAP, PROP_HF_PATH = 1, 2, 4
# rows of the properties table, in the reference's print order (tupsquantities.cpp:538-566)
PROPERTY_NAMES = ("Elec. Energy", "Real Elec. Energy", "Elec. + Nuc. Energy",
                  "NumberOfNegativeHessianEValues", "NumberOfNearZeroHessianEValues",
                  "NumberOfPositiveHessianEValues", "NumberOfNegativeHessianDiagValues",
                  "NumberOfNearZeroHessianDiagValues", "NumberOfPositiveHessianDiagValues",
                  "NumberOfPositiveMetricEValues", "NumberOfZeroMetricEValues", "NumberOfZeroMetricDiagonalValues",
                  "NormOfGradVector", "OverlapWithState_0 (re)", "OverlapWithState_0 (im)",
                  "MagOfOverlapWithState_0")
PROPERTY_ROWS = len(PROPERTY_NAMES)

_P = ctypes.c_void_p
_DP = ctypes.POINTER(ctypes.c_double)
_IP = ctypes.POINTER(ctypes.c_int)
_FP = ctypes.POINTER(ctypes.c_float)


class AegpuError(RuntimeError):
    pass


def lib(build_if_missing=True):
    """The loaded extension (builds it in-tree first if it is missing)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(LIB_PATH):
        if not build_if_missing:
            raise AegpuError("libansatzevolve_gb300.so is not built")
        from . import build as _b
        _b.build()
    L = ctypes.CDLL(LIB_PATH)
    i64 = ctypes.c_int64
    sig = {
        "aegpu_create": (ctypes.c_int, [ctypes.POINTER(_P)]),
        "aegpu_destroy": (None, [_P]),
        "aegpu_last_error": (ctypes.c_char_p, [_P]),
        "aegpu_set_problem": (ctypes.c_int, [_P] + [ctypes.c_int] * 7 + [_IP]),
        "aegpu_dim": (i64, [_P]),
        "aegpu_basis_states": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_uint32)]),
        "aegpu_num_blocks": (ctypes.c_int, [_P]),
        "aegpu_block_layout": (ctypes.c_int, [_P, _IP, _IP]),
        "aegpu_set_initial": (ctypes.c_int, [_P, _DP]),
        "aegpu_set_ham_csr": (ctypes.c_int, [_P, i64, ctypes.POINTER(i64), ctypes.POINTER(ctypes.c_int32), _DP]),
        "aegpu_set_ham_integrals": (ctypes.c_int, [_P, _DP, _DP, ctypes.c_int]),
        "aegpu_set_ham_integrals_batch": (ctypes.c_int, [_P, _DP, _DP, ctypes.c_int]),
        "aegpu_set_batch": (ctypes.c_int, [_P, ctypes.c_int]),
        "aegpu_batch_size": (ctypes.c_int, [_P]),
        "aegpu_set_active": (ctypes.c_int, [_P, _IP]),
        "aegpu_set_tuning": (ctypes.c_int, [_P, ctypes.c_int, ctypes.c_int]),
        "aegpu_flip_status": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_int)]),
        "aegpu_half_status": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_int)]),
        "aegpu_half_info": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_int64)]),
        "aegpu_get_tuning": (ctypes.c_int, [_P, ctypes.c_int]),
        "aegpu_io_dev": (ctypes.c_int, [_P, ctypes.POINTER(_P), ctypes.POINTER(_P), ctypes.POINTER(_P)]),
        "aegpu_io_put_angles": (ctypes.c_int, [_P, _DP, _P]),
        "aegpu_io_get_results": (ctypes.c_int, [_P, _DP, _DP, _P]),
        "aegpu_launch_io": (ctypes.c_int, [_P, _P]),
        "aegpu_optimise_newton": (ctypes.c_int, [_P, ctypes.c_int, _IP, _DP, _DP, ctypes.c_double, _DP, _DP,
                                                 ctypes.POINTER(i64), ctypes.POINTER(i64)]),
        "aegpu_optimise_batch": (ctypes.c_int, [_P, ctypes.c_int, _IP, _DP, _DP, ctypes.c_double, ctypes.c_int,
                                                ctypes.c_double, _DP, _DP, _DP, _IP, ctypes.POINTER(i64)]),
        "aegpu_mlp_create": (ctypes.c_int, [ctypes.POINTER(_P), ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                            ctypes.c_uint64]),
        "aegpu_mlp_destroy": (None, [_P]),
        "aegpu_mlp_last_error": (ctypes.c_char_p, [_P]),
        "aegpu_mlp_num_params": (i64, [_P]),
        "aegpu_mlp_set_scaling": (ctypes.c_int, [_P, _FP, _FP, _FP, _FP]),
        "aegpu_mlp_get_params": (ctypes.c_int, [_P, _FP]),
        "aegpu_mlp_set_params": (ctypes.c_int, [_P, _FP]),
        "aegpu_mlp_train": (ctypes.c_int, [_P, _FP, _FP, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_float,
                                           ctypes.c_uint64, _FP]),
        "aegpu_mlp_loss_grad": (ctypes.c_int, [_P, _FP, _FP, ctypes.c_int, _FP, _FP]),
        "aegpu_mlp_predict": (ctypes.c_int, [_P, _FP, ctypes.c_int, _FP]),
        "aegpu_mlp_predict_dev": (ctypes.c_int, [_P, _P, ctypes.c_int, _P, _P]),
        "aegpu_amplitude_width": (ctypes.c_int, [_P]),
        "aegpu_optimise_projected": (ctypes.c_int, [_P, ctypes.c_int, _IP, _DP, _DP, ctypes.c_double, ctypes.c_int,
                                                    _DP, _DP, ctypes.POINTER(i64), ctypes.POINTER(i64), _IP]),
        "aegpu_optimise_projected_diis": (ctypes.c_int, [_P, ctypes.c_int, _IP, _DP, _DP, ctypes.c_double,
                                                         ctypes.c_int, ctypes.c_int, ctypes.c_int, _DP, _DP,
                                                         ctypes.POINTER(i64), ctypes.POINTER(i64), _IP]),
        "aegpu_host_diis_coefficients": (ctypes.c_int, [ctypes.c_int, _DP, ctypes.c_int, _DP]),
        "aegpu_group_create": (ctypes.c_int, [ctypes.POINTER(_P), ctypes.POINTER(_P), ctypes.c_int]),
        "aegpu_group_launch": (ctypes.c_int, [_P, _P]),
        "aegpu_group_launch_count": (i64, [_P]),
        "aegpu_group_sync": (ctypes.c_int, [_P]),
        "aegpu_group_destroy": (None, [_P]),
        "aegpu_ham_info": (ctypes.c_int, [_P, _IP, ctypes.POINTER(i64)]),
        "aegpu_evolve": (ctypes.c_int, [_P, _DP, _DP]),
        "aegpu_energy": (ctypes.c_int, [_P, _DP, _DP]),
        "aegpu_gradient": (ctypes.c_int, [_P, _DP, _DP, _DP]),
        "aegpu_hessian": (ctypes.c_int, [_P, _DP, _IP, _DP, ctypes.c_int, _DP, _DP, _DP]),
        "aegpu_apply_h": (ctypes.c_int, [_P, _DP, _DP]),
        "aegpu_gradient_proj": (ctypes.c_int, [_P, _DP, _DP, _DP, _DP]),
        "aegpu_hessian_proj": (ctypes.c_int, [_P, _DP, _IP, _DP, ctypes.c_int, _DP, _DP, _DP, _DP]),
        "aegpu_hessian_metric": (ctypes.c_int, [_P, _DP, _IP, _DP, ctypes.c_int, _DP, _DP, _DP, _DP]),
        "aegpu_lowest_eigenpair": (ctypes.c_int, [_P, ctypes.c_double, ctypes.c_int, ctypes.c_int, _DP, _DP, _IP]),
        "aegpu_ground_state": (ctypes.c_int, [_P, _DP]),
        "aegpu_ground_overlap": (ctypes.c_int, [_P, _DP, _DP]),
        "aegpu_real_energy": (ctypes.c_int, [_P, _DP, _DP]),
        "aegpu_subspace_matrices": (ctypes.c_int, [_P, ctypes.c_int, _DP, _DP, _DP, _DP, _DP]),
        "aegpu_subspace_eigenvalues": (ctypes.c_int, [_P, ctypes.c_int, _DP, _DP, _IP]),
        "aegpu_host_tridiag_lowest": (ctypes.c_int, [ctypes.c_int, _DP, _DP, _DP, _DP]),
        "aegpu_host_subspace_eigenvalues": (ctypes.c_int, [ctypes.c_int, _DP, _DP, _DP, _DP, _DP, _IP]),
        "aegpu_path_properties": (ctypes.c_int, [_P, _DP, _IP, _DP, ctypes.c_int, ctypes.c_double, ctypes.c_int,
                                                 _DP, _DP, _DP]),
        "aegpu_gradient_dev": (ctypes.c_int, [_P, _P, _P, _P, _P]),
        "aegpu_energy_dev": (ctypes.c_int, [_P, _P, _P, _P]),
        "aegpu_state_dev": (ctypes.c_int, [_P, ctypes.POINTER(_P), ctypes.POINTER(_P)]),
        "aegpu_host_block_layout": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _IP, _IP, _IP, _IP]),
        "aegpu_host_half_orbits": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, _IP,
                                                  ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(ctypes.c_uint32),
                                                  ctypes.POINTER(i64), ctypes.POINTER(ctypes.c_uint32),
                                                  ctypes.POINTER(i64)]),
        "aegpu_host_pass_layout": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _IP, ctypes.c_int, ctypes.c_int, _IP, _IP,
                                                  _IP]),
        "aegpu_host_orbits": (ctypes.c_int, [ctypes.c_int] * 6 + [_IP, ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(i64),
                                                                  ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(i64),
                                                                  ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(i64)]),
        "aegpu_apply_dev": (ctypes.c_int, [_P, _P, _P, _P, _P]),
        "aegpu_use_graphs": (ctypes.c_int, [_P, ctypes.c_int]),
        "aegpu_csr_energy_noalloc": (ctypes.c_int, [i64, _P, _P, _P, _P, _P, _P, _P]),
        "aegpu_gram_upper_dev": (ctypes.c_int, [_P, i64, _P, i64, i64, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                                _P, _P, ctypes.c_int, _P]),
        "aegpu_exc_rule_dev": (ctypes.c_int, [ctypes.c_int, _IP, _P, i64, _P, _P, _P]),
        "aegpu_host_exc_rule": (ctypes.c_int, [ctypes.c_int, _IP, ctypes.POINTER(ctypes.c_uint32), i64,
                                               ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(ctypes.c_int8)]),
        "aegpu_phase_timing": (ctypes.c_int, [_P, ctypes.c_int]),
        "aegpu_phase_times": (ctypes.c_int, [_P, _DP, ctypes.POINTER(i64)]),
        "aegpu_problem_info": (ctypes.c_int, [_P, ctypes.POINTER(i64)]),
        "aegpu_device_bytes": (i64, [_P]),
        "aegpu_debug_fail_alloc_after": (None, [i64]),
        "aegpu_fp64_work": (ctypes.c_int, [_P, ctypes.POINTER(i64)]),
        "aegpu_fp64_peak": (ctypes.c_int, [_DP]),
        "aegpu_launch_count": (i64, [_P]),
        # reference C ABI
        "init": (_P, []),
        "cleanup": (ctypes.c_int, [_P]),
        "setExcitation": (ctypes.c_int, [ctypes.c_int, _IP, _IP, _P]),
        "setExcitationScale": (ctypes.c_int, [ctypes.c_int, _IP, _IP, _DP, _P]),
        "setHamiltonian": (ctypes.c_int, [ctypes.c_int, _IP, _IP, _DP, _P]),
        "setInitialState": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _IP, _DP, _P]),
        "setInitialStateComplex": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _IP, _DP, _P]),
        "getEnergy": (ctypes.c_int, [ctypes.c_int, _DP, _DP, _P]),
        "getFinalState": (ctypes.c_int, [ctypes.c_int, _DP, ctypes.c_int, _DP, _P]),
        "getFinalStateComplex": (ctypes.c_int, [ctypes.c_int, _DP, ctypes.c_int, _DP, _P]),
        "getGradient_COMP": (ctypes.c_int, [ctypes.c_int, _DP, _DP, _P]),
        "getHessian_COMP": (ctypes.c_int, [ctypes.c_int, _DP, _DP, _P]),
        "setTraceInterfaceCalls": (None, [ctypes.c_int]),
        "setRunPath": (ctypes.c_int, [ctypes.c_char_p, _P]),
        "setIntegrals": (ctypes.c_int, [ctypes.c_int, _DP, _DP, ctypes.c_int, _P]),
        "setNuclearEnergy": (ctypes.c_int, [ctypes.c_double, _P]),
        "optimise": (ctypes.c_int, [ctypes.c_int, _DP, _DP, _P]),
        "setRunFiles": (ctypes.c_int, [ctypes.c_char_p, _P]),
        "getExpectationValues": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _DP, _DP, _P]),
        "getProperties": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _DP, ctypes.c_int, _DP, _P]),
        "getLowestEigenvalue": (ctypes.c_int, [_DP, _DP, _P]),
        "writeProperties": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _DP, ctypes.c_int, ctypes.c_char_p, _P]),
        "setNumberOfOverlapsToCompute": (ctypes.c_int, [ctypes.c_int, _P]),
        "aegpu_host_tridiag_lowest_k": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _DP, _DP, _DP, _DP]),
        "aegpu_lowest_eigenpairs": (ctypes.c_int, [_P, ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_int, _DP,
                                                   _DP, _IP]),
        "aegpu_ground_overlaps": (ctypes.c_int, [_P, _DP, ctypes.c_int, _DP]),
        "getSubspaceEigenvalues": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _DP, _DP, _IP, _P]),
        # run-file readers (include/aegpu_runfiles.h)
        "aegpu_run_files_load": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_int, ctypes.POINTER(_P)]),
        "aegpu_run_files_error": (ctypes.c_char_p, []),
        "aegpu_run_files_sizes": (ctypes.c_int, [_P] + [_IP] * 6),
        "aegpu_run_files_get": (ctypes.c_int, [_P, _IP, _DP, _IP, _IP, _DP, _DP, _DP, _DP]),
        "aegpu_run_files_free": (None, [_P]),
        "aegpu_run_file_read": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_int, ctypes.POINTER(_P)]),
        "aegpu_run_files_parameters": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int,
                                                      ctypes.POINTER(_P)]),
        "generatePathsForSubspace": (ctypes.c_int, [ctypes.c_int, _DP, _IP, _DP, _P]),
        "iterativeOptimise": (ctypes.c_int, [ctypes.c_int, _DP, _DP, _P]),
        "getGradient": (ctypes.c_int, [ctypes.c_int, _DP, _DP, _P]),
        "getHessian": (ctypes.c_int, [ctypes.c_int, _DP, _DP, _P]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _LIB = L
    return L


def dptr(a):
    return a.ctypes.data_as(_DP)


def iptr(a):
    return a.ctypes.data_as(_IP)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


class Engine:
    """The aegpu C ABI for one problem (sector basis + excitations + Hamiltonian)."""

    def __init__(self, nq, basis_kind, n_elec, n_alpha, n_beta, ops0, complex_mode=False, tuning=None):
        self.L = lib()
        h = _P()
        rc = self.L.aegpu_create(ctypes.byref(h))
        if rc:
            raise AegpuError("aegpu_create failed (%d): no usable CUDA device" % rc)
        self.h = h
        # launch-shape knobs that must precede the problem set-up
        for knob in (TUNE_PASS_OPS, TUNE_CTAS_PER_SM):
            if tuning and knob in tuning:
                self._check(self.L.aegpu_set_tuning(h, knob, int(tuning[knob])))
        for knob in (TUNE_OTF_THREADS, TUNE_SPMV_TPR, TUNE_PDL):
            if tuning and knob in tuning:
                self._check(self.L.aegpu_set_tuning(h, knob, int(tuning[knob])))
        ops = _i32(ops0).reshape(-1, 4)
        self.nops = len(ops)
        self.W = 2 if complex_mode else 1
        self._check(self.L.aegpu_set_problem(h, nq, basis_kind, n_elec, n_alpha, n_beta, int(complex_mode), self.nops,
                                             iptr(ops.reshape(-1))))
        self.D = int(self.L.aegpu_dim(h))
        self.nb = 1

    def _check(self, rc):
        if rc:
            raise AegpuError("aegpu error %d: %s" % (rc, self.L.aegpu_last_error(self.h).decode()))

    def close(self):
        if getattr(self, "h", None):
            self.L.aegpu_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def states(self):
        out = np.zeros(self.D, dtype=np.uint32)
        self._check(self.L.aegpu_basis_states(self.h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))))
        return out

    def block_layout(self):
        nb = self.L.aegpu_num_blocks(self.h)
        perm = np.zeros(self.nops, dtype=np.int32)
        sizes = np.zeros(nb, dtype=np.int32)
        self._check(self.L.aegpu_block_layout(self.h, iptr(perm), iptr(sizes)))
        return perm, sizes

    def set_initial(self, amps):
        a = _f64(amps)
        assert a.size == self.D * self.W
        self._check(self.L.aegpu_set_initial(self.h, dptr(a)))

    def set_ham_csr(self, rowptr, col, val):
        rp = np.ascontiguousarray(rowptr, dtype=np.int64)
        c = np.ascontiguousarray(col, dtype=np.int32)
        v = _f64(val)
        self._check(self.L.aegpu_set_ham_csr(self.h, len(v), rp.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                                             c.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), dptr(v)))

    def set_ham_integrals(self, h1, g2, mode=HAM_AUTO):
        a, b = _f64(h1), _f64(g2)
        self._check(self.L.aegpu_set_ham_integrals(self.h, dptr(a), dptr(b), mode))

    def set_batch(self, nb):
        """Evaluate nb instances per call (angles [nb, nops] -> energies [nb], gradients [nb, nops])."""
        self._check(self.L.aegpu_set_batch(self.h, int(nb)))
        self.nb = int(self.L.aegpu_batch_size(self.h))

    def set_active(self, mask=None):
        """Skip instances with mask[b] == 0 in batched evaluations (None: all active)."""
        if mask is None:
            self._check(self.L.aegpu_set_active(self.h, None))
        else:
            m = _i32(mask)
            assert m.size == self.nb
            self._check(self.L.aegpu_set_active(self.h, iptr(m)))

    def set_ham_integrals_batch(self, h1s, g2s, mode=HAM_AUTO):
        """One Hamiltonian per instance: h1s [nb, N, N], g2s [nb, N, N, N, N]."""
        a, b = _f64(h1s), _f64(g2s)
        N2 = a.size // self.nb
        assert a.size == self.nb * N2 and b.size == self.nb * N2 * N2
        self._check(self.L.aegpu_set_ham_integrals_batch(self.h, dptr(a), dptr(b), mode))

    def _angles(self, angles_ops):
        a = _f64(angles_ops)
        assert a.size == self.nb * self.nops, "expected %d x %d angles" % (self.nb, self.nops)
        return a

    def ham_info(self):
        k = ctypes.c_int()
        n = ctypes.c_int64()
        self._check(self.L.aegpu_ham_info(self.h, ctypes.byref(k), ctypes.byref(n)))
        return k.value, n.value

    def evolve(self, angles_ops):
        a = self._angles(angles_ops)
        out = np.zeros(self.nb * self.D * self.W)
        self._check(self.L.aegpu_evolve(self.h, dptr(a), dptr(out)))
        return out if self.nb == 1 else out.reshape(self.nb, -1)

    def energy(self, angles_ops):
        a = self._angles(angles_ops)
        E = np.zeros(self.nb)
        self._check(self.L.aegpu_energy(self.h, dptr(a), dptr(E)))
        return E[0] if self.nb == 1 else E

    def gradient(self, angles_ops):
        a = self._angles(angles_ops)
        E = np.zeros(self.nb)
        g = np.zeros(self.nb * self.nops)
        self._check(self.L.aegpu_gradient(self.h, dptr(a), dptr(E), dptr(g)))
        if self.nb == 1:
            return E[0], g
        return E, g.reshape(self.nb, self.nops)

    def gradient_proj(self, angles_ops, proj):
        """(<proj|psi>, d<proj|psi>/dtheta_op) per instance (evolveDerivativeProj)."""
        a = self._angles(angles_ops)
        pr = _f64(proj)
        assert pr.size == self.nb * self.D * self.W
        ov = np.zeros(self.nb)
        g = np.zeros(self.nb * self.nops)
        self._check(self.L.aegpu_gradient_proj(self.h, dptr(a), dptr(pr), dptr(ov), dptr(g)))
        if self.nb == 1:
            return ov[0], g
        return ov, g.reshape(self.nb, self.nops)

    def hessian(self, angles_ops, param0, scale):
        a = _f64(angles_ops)
        p = _i32(param0)
        s = _f64(scale)
        P = int(p.max()) + 1
        E = np.zeros(1)
        g = np.zeros(P)
        H = np.zeros((P, P))
        self._check(self.L.aegpu_hessian(self.h, dptr(a), iptr(p), dptr(s), P, dptr(E), dptr(g), dptr(H)))
        return E[0], g, H

    def hessian_proj(self, angles_ops, param0, scale, proj):
        """(<proj|psi>, gradient, Hessian) of the overlap in the compressed parameters."""
        a = _f64(angles_ops)
        p = _i32(param0)
        s = _f64(scale)
        pr = _f64(proj)
        assert pr.size == self.D * self.W
        P = int(p.max()) + 1
        ov = np.zeros(1)
        g = np.zeros(P)
        H = np.zeros((P, P))
        self._check(self.L.aegpu_hessian_proj(self.h, dptr(a), iptr(p), dptr(s), P, dptr(pr), dptr(ov), dptr(g),
                                              dptr(H)))
        return ov[0], g, H

    def hessian_metric(self, angles_ops, param0, scale):
        """(E, gradient, Hessian, metric Re(T_C^dagger T_C)) in the compressed parameters."""
        a = _f64(angles_ops)
        p = _i32(param0)
        s = _f64(scale)
        P = int(p.max()) + 1
        E = np.zeros(1)
        g = np.zeros(P)
        H = np.zeros((P, P))
        M = np.zeros((P, P))
        self._check(self.L.aegpu_hessian_metric(self.h, dptr(a), iptr(p), dptr(s), P, dptr(E), dptr(g), dptr(H),
                                                dptr(M)))
        return E[0], g, H, M

    def lowest_eigenpair(self, tol=1e-8, basis=100, max_products=5000):
        """(eigenvalue, residual ||H v - lambda v||, H products) of the lowest eigenpair of
        H in the sector, by Lanczos from the initial state; the eigenvector stays on the
        device (ground_state, ground_overlap)."""
        lam, res = np.zeros(1), np.zeros(1)
        nprod = ctypes.c_int()
        self._check(self.L.aegpu_lowest_eigenpair(self.h, float(tol), int(basis), int(max_products), dptr(lam),
                                                  dptr(res), ctypes.byref(nprod)))
        return lam[0], res[0], nprod.value

    def lowest_eigenpairs(self, nstates, tol=1e-8, basis=100, max_products=20000):
        """(eigenvalues [nstates], residuals [nstates], H products) of the nstates lowest
        eigenpairs of H in the sector (every spin symmetry); the eigenvectors stay on the
        device (ground_overlaps)."""
        lam, res = np.zeros(nstates), np.zeros(nstates)
        nprod = ctypes.c_int()
        self._check(self.L.aegpu_lowest_eigenpairs(self.h, int(nstates), float(tol), int(basis), int(max_products),
                                                   dptr(lam), dptr(res), ctypes.byref(nprod)))
        return lam, res, nprod.value

    def ground_overlaps(self, angles_ops, nstates):
        """<psi(angles)|v_i> for the first nstates eigenvectors held (complex array)."""
        ov = np.zeros(2 * nstates)
        self._check(self.L.aegpu_ground_overlaps(self.h, dptr(self._angles(angles_ops)), int(nstates), dptr(ov)))
        return ov[0::2] + 1j * ov[1::2]

    def ground_state(self):
        v = np.zeros(self.D * self.W)
        self._check(self.L.aegpu_ground_state(self.h, dptr(v)))
        return v if self.W == 1 else v[0::2] + 1j * v[1::2]

    def ground_overlap(self, angles_ops):
        """<psi(angles)|v> with the lowest eigenvector (complex)."""
        ov = np.zeros(2)
        self._check(self.L.aegpu_ground_overlap(self.h, dptr(self._angles(angles_ops)), dptr(ov)))
        return complex(ov[0], ov[1])

    def real_energy(self, angles_ops):
        out = np.zeros(1)
        self._check(self.L.aegpu_real_energy(self.h, dptr(self._angles(angles_ops)), dptr(out)))
        return out[0]

    def subspace_matrices(self, angle_sets_ops):
        """(H, S): <psi_i|H|psi_j> and <psi_i|psi_j> of the states of the angle sets
        (complex arrays)."""
        a = _f64(np.atleast_2d(angle_sets_ops))
        n = a.shape[0]
        hr, hi, sr, si = (np.zeros((n, n)) for _ in range(4))
        self._check(self.L.aegpu_subspace_matrices(self.h, n, dptr(a), dptr(hr), dptr(hi), dptr(sr), dptr(si)))
        return hr + 1j * hi, sr + 1j * si

    def subspace_eigenvalues(self, angle_sets_ops):
        """(eigenvalues of S^-1/2 H S^-1/2, dimension of S's null space)."""
        a = _f64(np.atleast_2d(angle_sets_ops))
        w = np.zeros(a.shape[0])
        nr = ctypes.c_int()
        self._check(self.L.aegpu_subspace_eigenvalues(self.h, a.shape[0], dptr(a), dptr(w), ctypes.byref(nr)))
        return w, nr.value

    def path_properties(self, angles_ops, param0, scale, nuclear_energy=0.0, hessian=True, overlap=False):
        """One path's row of the properties table (PROPERTY_NAMES order, NaN where not
        computed), plus the Hessian and metric when `hessian`."""
        a = self._angles(angles_ops)
        p = _i32(param0)
        s = _f64(scale)
        P = int(p.max()) + 1
        row = np.zeros(PROPERTY_ROWS)
        H = np.zeros((P, P))
        M = np.zeros((P, P))
        flags = (PROP_HESSIAN if hessian else 0) | (PROP_OVERLAP if overlap else 0)
        self._check(self.L.aegpu_path_properties(self.h, dptr(a), iptr(p), dptr(s), P, float(nuclear_energy), flags,
                                                 dptr(row), dptr(H), dptr(M)))
        return row, (H if hessian else None), (M if hessian else None)

    def apply_h(self, x):
        x = _f64(x)
        assert x.size == self.nb * self.D * self.W
        y = np.zeros_like(x)
        self._check(self.L.aegpu_apply_h(self.h, dptr(x), dptr(y)))
        return y

    def gradient_dev(self, angles_ptr, energy_ptr, grad_ptr, stream=0):
        self._check(self.L.aegpu_gradient_dev(self.h, angles_ptr, energy_ptr, grad_ptr, stream or None))

    def energy_dev(self, angles_ptr, energy_ptr, stream=0):
        self._check(self.L.aegpu_energy_dev(self.h, angles_ptr, energy_ptr, stream or None))

    def apply_dev(self, x_ptr, y_ptr, energy_ptr=None, stream=0):
        self._check(self.L.aegpu_apply_dev(self.h, x_ptr, y_ptr, energy_ptr, stream or None))

    def io_dev(self):
        """Device addresses (angles [nb, nops], energies [nb], gradients [nb, nops]) that
        the captured evaluation graph reads and writes."""
        a, e, g = _P(), _P(), _P()
        self._check(self.L.aegpu_io_dev(self.h, ctypes.byref(a), ctypes.byref(e), ctypes.byref(g)))
        return a.value, e.value, g.value

    def io_put_angles(self, angles_ops, stream=0):
        a = self._angles(angles_ops)
        self._io_keep = a  # the copy is asynchronous: keep the host array alive
        self._check(self.L.aegpu_io_put_angles(self.h, dptr(a), stream or None))

    def io_get_results(self, stream=0):
        E = np.zeros(self.nb)
        g = np.zeros(self.nb * self.nops)
        self._check(self.L.aegpu_io_get_results(self.h, dptr(E), dptr(g), stream or None))
        return E, g.reshape(self.nb, self.nops)

    def launch_io(self, stream=0):
        self._check(self.L.aegpu_launch_io(self.h, stream or None))

    def optimise_newton(self, x0, param0, scale, gtol=1e-6):
        """The reference's Newton method on this (batch-of-1) engine: (x, E, |g|, hessian evals, energy evals)."""
        x = _f64(x0).copy()
        p, s = _i32(param0), _f64(scale)
        E, gn = np.zeros(1), np.zeros(1)
        nh, ne = ctypes.c_int64(), ctypes.c_int64()
        self._check(self.L.aegpu_optimise_newton(self.h, len(x), iptr(p), dptr(s), dptr(x), gtol, dptr(E), dptr(gn),
                                                 ctypes.byref(nh), ctypes.byref(ne)))
        return x, E[0], gn[0], nh.value, ne.value

    def optimise_projected(self, x0, param0, scale, gtol=1e-5, max_outer=3000, diis=0, ediis=True):
        """The reference's projected iteration (iterativeTups): (x, E, |g_proj|, Hessians,
        evaluations, renewals).  diis > 0 extrapolates the angles over that many renewals
        (EDIIS, or Pulay DIIS with ediis=False); the reference ships it off (0)."""
        x = _f64(x0).copy()
        p, s = _i32(param0), _f64(scale)
        E, gn = np.zeros(1), np.zeros(1)
        nh, ne = ctypes.c_int64(), ctypes.c_int64()
        it = ctypes.c_int()
        self._check(self.L.aegpu_optimise_projected_diis(self.h, len(x), iptr(p), dptr(s), dptr(x), gtol,
                                                         int(max_outer), int(diis), int(bool(ediis)), dptr(E),
                                                         dptr(gn), ctypes.byref(nh), ctypes.byref(ne),
                                                         ctypes.byref(it)))
        return x, E[0], gn[0], nh.value, ne.value, it.value

    def optimise_batch(self, x0, param0, scale, gtol=1e-6, max_rounds=2000, max_step=1.0, hinv=None):
        """Lockstep BFGS of all instances from x0 [nb, P]: (x, E [nb], |g| [nb], iterations [nb], rounds).
        hinv [nb, P, P] (optional): initial inverse Hessians, overwritten with the final ones."""
        x = _f64(x0).reshape(self.nb, -1).copy()
        P = x.shape[1]
        p, s = _i32(param0), _f64(scale)
        E, gn = np.zeros(self.nb), np.zeros(self.nb)
        it = np.zeros(self.nb, dtype=np.int32)
        r = ctypes.c_int64()
        hp = None
        if hinv is not None:
            assert hinv.dtype == np.float64 and hinv.flags.c_contiguous and hinv.size == self.nb * P * P
            hp = dptr(hinv)
        self._check(self.L.aegpu_optimise_batch(self.h, P, iptr(p), dptr(s), dptr(x), gtol, int(max_rounds), max_step,
                                                hp, dptr(E), dptr(gn), iptr(it), ctypes.byref(r)))
        return x, E, gn, it, r.value

    def tuning(self):
        return {k: int(self.L.aegpu_get_tuning(self.h, k))
                for k in (TUNE_PASS_OPS, TUNE_CTAS_PER_SM, TUNE_OTF_THREADS, TUNE_SPMV_TPR, TUNE_PDL)}

    def set_tuning(self, knob, value):
        """One knob (TUNE_*) where the engine accepts it at this point of its set-up
        (TUNE_PDL, TUNE_REUSE_HPSI, TUNE_FLIP and TUNE_HALF at any time)."""
        self._check(self.L.aegpu_set_tuning(self.h, knob, int(value)))

    def get_tuning(self, knob):
        return int(self.L.aegpu_get_tuning(self.h, knob))

    def flip_status(self):
        """Per instance: True where the last energy evaluation's H psi took the spin-flip
        half product."""
        u = np.zeros(self.nb, dtype=np.int32)
        self._check(self.L.aegpu_flip_status(self.h, iptr(u)))
        return u.astype(bool)

    def half_status(self):
        """Per instance: True where the last evaluation ran the spin-flip half passes."""
        u = np.zeros(self.nb, dtype=np.int32)
        self._check(self.L.aegpu_half_status(self.h, iptr(u)))
        return u.astype(bool)

    def half_info(self):
        """Whether the problem allows the spin-flip half passes, the amplitudes they touch
        per sweep and the FP64 instructions of their forward and adjoint passes."""
        out = np.zeros(4, dtype=np.int64)
        self._check(self.L.aegpu_half_info(self.h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))))
        return {"available": bool(out[0]), "active": int(out[1]), "fwd_fp64": int(out[2]), "adj_fp64": int(out[3])}

    def use_graphs(self, enable=True):
        self._check(self.L.aegpu_use_graphs(self.h, int(enable)))

    def phase_timing(self, enable=True):
        self._check(self.L.aegpu_phase_timing(self.h, int(enable)))

    def phase_times(self):
        ms = np.zeros(3)
        n = ctypes.c_int64()
        self._check(self.L.aegpu_phase_times(self.h, dptr(ms), ctypes.byref(n)))
        return ms, n.value

    def info(self):
        out = np.zeros(8, dtype=np.int64)
        self._check(self.L.aegpu_problem_info(self.h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))))
        keys = ("D", "nops", "blocks", "ham_kind", "ham_entries", "ell_width", "active", "nnz")
        return dict(zip(keys, map(int, out)))

    def fp64_work(self, half=None, half_passes=None):
        """FP64 instructions per evaluation and instance: (H psi, forward, adjoint).  H psi
        counts the spin-flip half product where half is true, the full product where it
        is false, and by default what the last energy evaluation took (averaged over
        the instances); the passes likewise the spin-flip half passes (half_passes)."""
        w = np.zeros(4, dtype=np.int64)
        self._check(self.L.aegpu_fp64_work(self.h, w.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))))
        frac = float(np.mean(self.flip_status())) if half is None else float(bool(half))
        hpsi = int(round(w[0] * (1.0 - frac) + w[3] * frac))
        hi = self.half_info()
        pf = 0.0
        if hi["available"]:
            pf = float(np.mean(self.half_status())) if half_passes is None else float(bool(half_passes))
        fwd = int(round(w[1] * (1.0 - pf) + hi["fwd_fp64"] * pf))
        adj = int(round(w[2] * (1.0 - pf) + hi["adj_fp64"] * pf))
        return hpsi, fwd, adj

    def device_bytes(self):
        return int(self.L.aegpu_device_bytes(self.h))

    def launch_count(self):
        return int(self.L.aegpu_launch_count(self.h))


class Group:
    """Several engines evaluated by one CUDA graph launch (aegpu_group_*)."""

    def __init__(self, engines):
        self.L = lib()
        self.engines = list(engines)
        arr = (_P * len(self.engines))(*[e.h for e in self.engines])
        h = _P()
        rc = self.L.aegpu_group_create(ctypes.byref(h), arr, len(self.engines))
        if rc:
            msgs = "; ".join(self.L.aegpu_last_error(e.h).decode() for e in self.engines)
            raise AegpuError("aegpu_group_create failed (%d): %s" % (rc, msgs))
        self.h = h

    def launch(self, stream=0):
        rc = self.L.aegpu_group_launch(self.h, stream or None)
        if rc:
            msgs = "; ".join(self.L.aegpu_last_error(e.h).decode() for e in self.engines)
            raise AegpuError("aegpu_group_launch failed (%d): %s" % (rc, msgs))

    def sync(self):
        if self.L.aegpu_group_sync(self.h):
            raise AegpuError("aegpu_group_sync failed")

    def launch_count(self):
        return int(self.L.aegpu_group_launch_count(self.h))

    def close(self):
        if getattr(self, "h", None):
            self.L.aegpu_group_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()


def fp64_peak():
    """Measured DFMA throughput of the current CUDA device in TFLOP/s."""
    t = ctypes.c_double()
    rc = lib().aegpu_fp64_peak(ctypes.byref(t))
    if rc:
        raise AegpuError("aegpu_fp64_peak failed (%d)" % rc)
    return t.value


def host_block_layout(nq, ops0):
    """Operator application order and fused block sizes (host setup, no GPU)."""
    L = lib()
    ops = _i32(ops0).reshape(-1, 4)
    perm = np.zeros(len(ops), dtype=np.int32)
    sizes = np.zeros(len(ops), dtype=np.int32)
    nb = ctypes.c_int(len(ops))
    rc = L.aegpu_host_block_layout(nq, len(ops), iptr(ops.reshape(-1)), iptr(perm), iptr(sizes), ctypes.byref(nb))
    if rc:
        raise AegpuError("aegpu_host_block_layout returned %d" % rc)
    return perm, sizes[:nb.value]


def host_orbits(nq, kind, ne, na, nb, ops0):
    """Orbit tables of one block of commuting excitations (host setup, no GPU):
    (ranks, groups[:, idx_off n_orbits k mask], tiles[:, group orbit0 n_orbits elem_off])."""
    L = lib()
    ops = _i32(ops0).reshape(-1, 4)
    u32 = ctypes.POINTER(ctypes.c_uint32)
    ni, ng, nt = ctypes.c_int64(0), ctypes.c_int64(0), ctypes.c_int64(0)
    args = [nq, kind, ne, na, nb, len(ops), iptr(ops.reshape(-1))]
    rc = L.aegpu_host_orbits(*args, None, ctypes.byref(ni), None, ctypes.byref(ng), None, ctypes.byref(nt))
    if rc:
        raise AegpuError("aegpu_host_orbits returned %d" % rc)
    idx = np.zeros(ni.value, dtype=np.uint32)
    g = np.zeros((ng.value, 4), dtype=np.uint32)
    t = np.zeros((nt.value, 4), dtype=np.uint32)
    rc = L.aegpu_host_orbits(*args, idx.ctypes.data_as(u32), ctypes.byref(ni), g.ctypes.data_as(u32), ctypes.byref(ng),
                             t.ctypes.data_as(u32), ctypes.byref(nt))
    if rc:
        raise AegpuError("aegpu_host_orbits returned %d" % rc)
    return idx, g, t


def host_pass_layout(nq, ops0, max_pass=6, mirror_split=False):
    """The engine's passes (host setup, no GPU): (list of operator arrays, diagonal flags,
    mirror cut applied)."""
    L = lib()
    ops = _i32(ops0).reshape(-1, 4)
    n = ctypes.c_int(len(ops) + 1)
    po = np.zeros(len(ops), dtype=np.int32)
    ps = np.zeros(len(ops) + 1, dtype=np.int32)
    rc = L.aegpu_host_pass_layout(nq, len(ops), iptr(ops.reshape(-1)), max_pass, int(mirror_split), iptr(po), iptr(ps),
                                  ctypes.byref(n))
    if rc not in (0, 5):  # 5: AEGPU_ERR_UNSUPPORTED (no mirror cut)
        raise AegpuError("aegpu_host_pass_layout returned %d" % rc)
    passes, diag, k = [], [], 0
    for sz in ps[:n.value]:
        passes.append(po[k:k + abs(int(sz))].copy())
        diag.append(sz < 0)
        k += abs(int(sz))
    return passes, diag, rc == 0 and bool(mirror_split)


def host_half_orbits(nq, n_alpha, ops0):
    """Spin-flip half tables of one pass (host setup, no GPU): (ranks, bitstrings,
    tasks[:, group elem_off n mask]); AegpuError where the pass has no mirror symmetry."""
    L = lib()
    ops = _i32(ops0).reshape(-1, 4)
    u32 = ctypes.POINTER(ctypes.c_uint32)
    ni, nt = ctypes.c_int64(0), ctypes.c_int64(0)
    args = [nq, n_alpha, len(ops), iptr(ops.reshape(-1))]
    rc = L.aegpu_host_half_orbits(*args, None, None, ctypes.byref(ni), None, ctypes.byref(nt))
    if rc:
        raise AegpuError("aegpu_host_half_orbits returned %d" % rc)
    idx = np.zeros(ni.value, dtype=np.uint32)
    bits = np.zeros(ni.value, dtype=np.uint32)
    t = np.zeros((nt.value, 4), dtype=np.uint32)
    rc = L.aegpu_host_half_orbits(*args, idx.ctypes.data_as(u32), bits.ctypes.data_as(u32), ctypes.byref(ni),
                                  t.ctypes.data_as(u32), ctypes.byref(nt))
    if rc:
        raise AegpuError("aegpu_host_half_orbits returned %d" % rc)
    return idx, bits, t


class stateAnsatzManager:
    """Python mirror of the reference binding (PyAnsatzEvolve.cpp:17-148) over the
    C ABI: same method names, 1-based operators for storeOperators, 0-based
    indices for storeInitial / storeHamiltonian, compressed or per-operator angles."""

    def __init__(self):
        self.L = lib()
        self.ctx = _P(self.L.init())
        self._ops = None
        self._order = None
        self._nq = None
        self._P = None
        self._angles = None

    def close(self):
        if getattr(self, "ctx", None) is not None and self.ctx.value:
            self.L.cleanup(ctypes.byref(self.ctx))

    def __del__(self):
        self.close()

    def _push_excitations(self):
        if self._ops is None or self._order is None:
            return True
        ops = np.asarray(self._ops, dtype=np.int32).reshape(-1, 4)
        n = len(ops)
        fortran = _i32(ops.T.reshape(-1))  # operators[n*j + i]
        order = _i32([o[0] + 1 for o in self._order])
        scale = _f64([o[1] for o in self._order])
        if len(order) != n:
            return False
        return self.L.setExcitationScale(n, iptr(fortran), iptr(order), dptr(scale), self.ctx) == 0

    def storeOperators(self, operators):
        self._ops = [list(map(int, o)) for o in operators]
        if any(len(o) != 4 for o in self._ops):
            raise ValueError("Operator must be 4 long")
        return self._push_excitations()

    def storeParameterDependencies(self, dep):
        self._order = [(int(p), float(s)) for p, s in dep]
        self._P = max(p for p, _ in self._order) + 1
        return self._push_excitations()

    def storeInitial(self, numberOfQubits, indexes, coeffs):
        idx = _i32(np.asarray(indexes) + 1)
        c = np.asarray(coeffs)
        self._nq = int(numberOfQubits)
        if np.iscomplexobj(c):
            cc = np.ascontiguousarray(c, dtype=np.complex128)
            return self.L.setInitialStateComplex(self._nq, len(idx), iptr(idx), cc.ctypes.data_as(_DP), self.ctx) == 0
        return self.L.setInitialState(self._nq, len(idx), iptr(idx), dptr(_f64(c)), self.ctx) == 0

    def storeHamiltonian(self, iIndexes, jIndexes, coeffs):
        i = _i32(np.asarray(iIndexes) + 1)
        j = _i32(np.asarray(jIndexes) + 1)
        return self.L.setHamiltonian(len(i), iptr(i), iptr(j), dptr(_f64(coeffs)), self.ctx) == 0

    def storeNuclearEnergy(self, e):
        return self.L.setNuclearEnergy(float(e), self.ctx) == 0

    def storeRunPath(self, path):
        return self.L.setRunPath(path.encode(), self.ctx) == 0

    def storeRunFiles(self, prefix):
        """The whole setup the reference's driver reads from `prefix` (initial state,
        operators, order, nuclear energy, Hamiltonian files); returns the loaded
        ``runfiles.RunFiles`` (its parameter_sets are the file's angle sets)."""
        from .runfiles import load_run_files
        rf = load_run_files(prefix)
        if self.L.setRunFiles(prefix.encode(), self.ctx) != 0:
            raise AegpuError("setRunFiles refused " + prefix)
        self._nq = rf.nq
        self._ops = [list(map(int, o)) for o in rf.operators]
        self._order = [(int(p), float(c)) for p, c in zip(rf.order, rf.scale)]
        self._P = rf.n_params
        return rf

    def storeIntegrals(self, h1, g2, mode=HAM_AUTO):
        h1 = _f64(h1)
        return self.L.setIntegrals(h1.shape[0], dptr(h1), dptr(_f64(g2)), mode, self.ctx) == 0

    # current angles (setAngles / getAngles, AnsatzManager.cpp:467-506): the getters
    # without angles evaluate at them, the getters with angles set them first
    def setAngles(self, angles):
        a = _f64(angles).copy()
        n_ops = len(self._ops) if self._ops is not None else None
        if self._P is not None and n_ops is not None and a.size not in (self._P, n_ops):
            return False
        self._angles = a
        return True

    def getAngles(self):
        """The current angles, compressed (the first operator of each parameter divided
        by its scale when per-operator angles were set)."""
        a = self._current(None)
        if self._order is None or a.size == self._P:
            return a.copy()
        x = np.zeros(self._P)
        seen = np.zeros(self._P, dtype=bool)
        for o, (p, c) in enumerate(self._order):
            if not seen[p] and c != 0:
                x[p], seen[p] = a[o] / c, True
        return x

    def _current(self, angles):
        if angles is not None:
            if not self.setAngles(angles):
                raise AegpuError("Incorrect number of angles given %d" % np.size(angles))
        if getattr(self, "_angles", None) is None:
            raise AegpuError("no angles set")
        return self._angles

    def _per_op(self, a):
        return self._ops is not None and self._P is not None and a.size == len(self._ops) and a.size != self._P

    def getExpectationValue(self, angles=None):
        a = self._current(angles)
        E = np.zeros(1)
        rc = self.L.getEnergy(len(a), dptr(a), dptr(E), self.ctx)
        if rc:
            raise AegpuError("getEnergy returned %d" % rc)
        return E[0]

    def getFinalState(self, angles=None, complex_state=False):
        a = self._current(angles)
        n = 1 << self._nq
        if complex_state:
            out = np.zeros(n, dtype=np.complex128)
            rc = self.L.getFinalStateComplex(len(a), dptr(a), n, out.ctypes.data_as(_DP), self.ctx)
        else:
            out = np.zeros(n)
            rc = self.L.getFinalState(len(a), dptr(a), n, dptr(out), self.ctx)
        if rc:
            raise AegpuError("getFinalState returned %d" % rc)
        return out

    def getGradient(self, angles=None):
        """Derivatives with respect to every operator's angle (the reference's fused build
        traps here; every operator is its own parameter)."""
        a = self._current(angles)
        g = np.zeros(len(self._ops))
        rc = self.L.getGradient(len(a), dptr(a), dptr(g), self.ctx)
        if rc:
            raise AegpuError("getGradient returned %d" % rc)
        return g

    def getHessian(self, angles=None):
        a = self._current(angles)
        n = len(self._ops)
        H = np.zeros(n * n)
        rc = self.L.getHessian(len(a), dptr(a), dptr(H), self.ctx)
        if rc:
            raise AegpuError("getHessian returned %d" % rc)
        return H.reshape(n, n)

    def _compress_rows(self):
        C = np.zeros((self._P, len(self._order)))
        for o, (p, c) in enumerate(self._order):
            C[p, o] = c
        return C

    def getGradientComp(self, angles=None):
        a = self._current(angles)
        if self._per_op(a):  # the C entry point takes compressed angles only
            return self._compress_rows() @ self.getGradient()
        g = np.zeros(len(a))
        rc = self.L.getGradient_COMP(len(a), dptr(a), dptr(g), self.ctx)
        if rc:
            raise AegpuError("getGradient_COMP returned %d" % rc)
        return g

    def getHessianComp(self, angles=None):
        a = self._current(angles)
        if self._per_op(a):
            C = self._compress_rows()
            return C @ self.getHessian() @ C.T
        H = np.zeros(len(a) * len(a))
        rc = self.L.getHessian_COMP(len(a), dptr(a), dptr(H), self.ctx)
        if rc:
            raise AegpuError("getHessian_COMP returned %d" % rc)
        return H.reshape(len(a), len(a), order="F")

    def getExpectationValues(self, angles):
        """Energies of the angle rows (compressed or per operator), one batched GPU
        evaluation (evolveMultiple + getEnergies in the reference)."""
        a = _f64(np.atleast_2d(angles))
        E = np.zeros(a.shape[0])
        rc = self.L.getExpectationValues(a.shape[0], a.shape[1], dptr(a), dptr(E), self.ctx)
        if rc:
            raise AegpuError("getExpectationValues returned %d" % rc)
        return E

    def getProperties(self, paths, hessian=True, overlap=True):
        """writeProperties' table: {row name: values per path} (PROPERTY_NAMES rows, NaN
        where not computed)."""
        a = _f64(np.atleast_2d(paths))
        t = np.zeros((a.shape[0], PROPERTY_ROWS))
        flags = (PROP_HESSIAN if hessian else 0) | (PROP_OVERLAP if overlap else 0)
        rc = self.L.getProperties(a.shape[0], a.shape[1], dptr(a), flags, dptr(t), self.ctx)
        if rc:
            raise AegpuError("getProperties returned %d" % rc)
        return {name: t[:, k] for k, name in enumerate(PROPERTY_NAMES)}

    def iterativeOptimise(self, angles=None):
        """The projected iteration (iterativeTups) then Newton-Raphson from the given (or
        current) angles; returns (energy, compressed angles), which become current."""
        a = _f64(self._current(angles)).copy()
        E = np.zeros(1)
        rc = self.L.iterativeOptimise(len(a), dptr(a), dptr(E), self.ctx)
        if rc:
            raise AegpuError("iterativeOptimise returned %d" % rc)
        self._angles = a.copy()
        return E[0], a

    def generatePathsForSubspace(self, numberOfPaths):
        """Distinct minima from seeded random starts and the subspace diagonalisation over
        them: (eigenvalues, overlap null rank, minima energies with the nuclear energy)."""
        n = int(numberOfPaths)
        w, E = np.zeros(n), np.zeros(n)
        nr = ctypes.c_int()
        rc = self.L.generatePathsForSubspace(n, dptr(w), ctypes.byref(nr), dptr(E), self.ctx)
        if rc:
            raise AegpuError("generatePathsForSubspace returned %d" % rc)
        return w, nr.value, E

    def writeProperties(self, paths, runPath=None, hessian=True, overlap=True, hf_path=True):
        """The reference's writeProperties output: its table on stdout and, with a run
        path, the per-path Hessian / metric files and the ground-state overlap vector."""
        a = _f64(np.atleast_2d(paths))
        flags = (PROP_HESSIAN if hessian else 0) | (PROP_OVERLAP if overlap else 0) | (PROP_HF_PATH if hf_path else 0)
        rc = self.L.writeProperties(a.shape[0], a.shape[1], dptr(a), flags,
                                    None if runPath is None else str(runPath).encode(), self.ctx)
        if rc:
            raise AegpuError("writeProperties returned %d" % rc)

    def setNumberOfOverlapsToCompute(self, n):
        """The reference's numberOfOverlapsToCompute option of writeProperties: overlaps
        with the n lowest eigenstates when H has fewer than 5,000 rows, else the lowest."""
        rc = self.L.setNumberOfOverlapsToCompute(int(n), self.ctx)
        if rc:
            raise AegpuError("setNumberOfOverlapsToCompute returned %d" % rc)
        return True

    def getLowestEigenvalue(self):
        """(lowest eigenvalue of H in the sector, without the nuclear energy; residual)."""
        E, r = np.zeros(1), np.zeros(1)
        rc = self.L.getLowestEigenvalue(dptr(E), dptr(r), self.ctx)
        if rc:
            raise AegpuError("getLowestEigenvalue returned %d" % rc)
        return E[0], r[0]

    def getSubspaceEigenvalues(self, paths):
        a = _f64(np.atleast_2d(paths))
        w = np.zeros(a.shape[0])
        nr = ctypes.c_int()
        rc = self.L.getSubspaceEigenvalues(a.shape[0], a.shape[1], dptr(a), dptr(w), ctypes.byref(nr), self.ctx)
        if rc:
            raise AegpuError("getSubspaceEigenvalues returned %d" % rc)
        return w, nr.value

    def optimise(self, angles=None):
        """Newton-Raphson from the given (or current) angles; returns (energy, optimised
        compressed angles) and makes them the current angles (the reference binding's
        optimise() returns only its success flag)."""
        a = _f64(self._current(angles)).copy()
        E = np.zeros(1)
        rc = self.L.optimise(len(a), dptr(a), dptr(E), self.ctx)
        if rc:
            raise AegpuError("optimise returned %d" % rc)
        self._angles = a.copy()
        return E[0], a


# the reference binding's module functions (file readers), at package level as there
from .runfiles import loadNuclearEnergy, loadOperators, loadParameters, loadPath, readCsvState  # noqa: E402,F401
