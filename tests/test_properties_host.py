"""Host parts of the properties entry points, on the CPU: the tridiagonal eigen-solve
inside the Lanczos iteration (aegpu_host_tridiag_lowest) against numpy, including
clustered, degenerate and badly scaled spectra."""
import numpy as np
import pytest

from ansatzevolve_gb300 import dptr, lib


def _solve(a, b):
    k = len(a)
    v = np.zeros(k)
    th = np.zeros(1)
    assert lib().aegpu_host_tridiag_lowest(k, dptr(np.ascontiguousarray(a, dtype=float)),
                                           dptr(np.ascontiguousarray(b if k > 1 else [0.0], dtype=float)),
                                           dptr(v), dptr(th)) == 0
    return th[0], v


@pytest.mark.parametrize("k,seed,scale", [(1, 0, 1.0), (2, 1, 1.0), (7, 2, 1.0), (60, 3, 1.0), (150, 4, 1e3),
                                          (40, 5, 1e-6)])
def test_tridiagonal_lowest_eigenpair(k, seed, scale):
    rng = np.random.default_rng(seed)
    a = rng.normal(size=k) * scale
    b = rng.normal(size=k - 1) * scale
    T = np.diag(a) + np.diag(b, 1) + np.diag(b, -1)
    w, V = np.linalg.eigh(T)
    th, v = _solve(a, b)
    assert abs(th - w[0]) <= 1e-13 * np.abs(w).max()
    assert abs(np.linalg.norm(v) - 1.0) < 1e-13
    assert np.linalg.norm(T @ v - th * v) <= 1e-10 * np.abs(w).max()


def test_tridiagonal_with_tiny_couplings_and_clusters():
    # a Lanczos matrix near convergence: tiny off-diagonals and a near-degenerate bottom
    a = np.array([-3.0, -3.0 + 1e-9, -1.0, 0.5, 2.0])
    b = np.array([1e-12, 1e-6, 0.3, 0.0])
    T = np.diag(a) + np.diag(b, 1) + np.diag(b, -1)
    w = np.linalg.eigvalsh(T)
    th, v = _solve(a, b)
    assert abs(th - w[0]) < 1e-14
    assert np.linalg.norm(T @ v - th * v) < 1e-10


@pytest.mark.parametrize("cplx", [False, True])
def test_subspace_eigen_analysis_matches_numpy(cplx):
    """S^-1/2 H S^-1/2 with a rank-deficient overlap matrix (two states repeated): the
    null space gives eigenvalue 0 (doSubspaceDiagonalisation keeps it) and its rank is
    reported."""
    import ctypes
    rng = np.random.default_rng(7)
    D, n = 30, 6
    X = rng.normal(size=(D, n - 2)) + (1j * rng.normal(size=(D, n - 2)) if cplx else 0)
    X = np.column_stack([X, X[:, 0], X[:, 1]])
    X /= np.linalg.norm(X, axis=0)  # unit states, as evolved states are
    A = rng.normal(size=(D, D)) + (1j * rng.normal(size=(D, D)) if cplx else 0)
    Hd = 0.5 * (A + A.conj().T)
    S = X.conj().T @ X
    H = X.conj().T @ Hd @ X
    ws, Vs = np.linalg.eigh(S)
    f = np.where(ws < 1e-14, 0.0, 1 / np.sqrt(np.abs(ws)))
    Y = (Vs * f) @ Vs.conj().T @ H @ (Vs * f) @ Vs.conj().T
    want = np.linalg.eigvalsh(0.5 * (Y + Y.conj().T))
    w = np.zeros(n)
    nr = ctypes.c_int()
    c = lambda M: dptr(np.ascontiguousarray(M, dtype=float))  # noqa: E731
    hr, hi, sr, si = H.real.copy(), H.imag.copy(), S.real.copy(), S.imag.copy()
    assert lib().aegpu_host_subspace_eigenvalues(n, c(hr), c(hi), c(sr), c(si), dptr(w), ctypes.byref(nr)) == 0
    assert nr.value == int((ws < 1e-14).sum()) == 2
    np.testing.assert_allclose(w, want, atol=1e-9 * np.abs(want).max(), rtol=0)


def test_properties_c_abi_status_codes():
    import ctypes
    L = lib()
    a = np.zeros(4)
    t = np.zeros(64)
    nr = ctypes.c_int()
    assert L.getProperties(1, 4, dptr(a), 3, dptr(t), None) == 1
    assert L.getLowestEigenvalue(dptr(a), dptr(a), None) == 1
    assert L.getSubspaceEigenvalues(1, 4, dptr(a), dptr(a), ctypes.byref(nr), None) == 1
    ctx = ctypes.c_void_p(L.init())
    try:
        assert L.getProperties(0, 4, dptr(a), 3, dptr(t), ctx) == 2
        assert L.getProperties(1, 4, dptr(a), 3, None, ctx) == 2
        assert L.getLowestEigenvalue(None, None, ctx) == 2
        assert L.getSubspaceEigenvalues(1, 0, dptr(a), dptr(a), ctypes.byref(nr), ctx) == 2
        # nothing set up: the first evaluation fails cleanly (no GPU work happens)
        assert L.getProperties(1, 4, dptr(a), 3, dptr(t), ctx) == 3
    finally:
        L.cleanup(ctypes.byref(ctx))


@pytest.mark.parametrize("ediis", [False, True])
@pytest.mark.parametrize("n,seed", [(1, 0), (3, 1), (8, 2), (15, 3)])
def test_diis_coefficients_match_restatement(ediis, n, seed):
    """The DIIS step of the projected iteration (aegpu_host_diis_coefficients) against
    the numpy restatement of diis.h / diis.cpp, on Gram matrices of error vectors."""
    from oracle.diis_ref import ediis as ediis_ref, pulay
    rng = np.random.default_rng(seed)
    E = rng.normal(size=(n, 40)) * np.geomspace(1, 1e-3, n)[:, None]  # shrinking errors
    B = E @ E.T
    c = np.zeros(n)
    assert lib().aegpu_host_diis_coefficients(n, dptr(np.ascontiguousarray(B)), int(ediis), dptr(c)) == 0
    want = ediis_ref(B) if ediis else pulay(B)
    np.testing.assert_allclose(c, want, atol=1e-9, rtol=0)
    if not ediis:
        assert abs(c.sum() - 1) < 1e-12
    else:
        assert (c >= 0).all()


def test_pulay_with_rank_deficient_errors():
    from oracle.diis_ref import pulay
    rng = np.random.default_rng(9)
    e = rng.normal(size=(3, 20))
    E = np.vstack([e, e[0] + e[1]])  # four errors spanning three directions
    B = E @ E.T
    c = np.zeros(4)
    assert lib().aegpu_host_diis_coefficients(4, dptr(np.ascontiguousarray(B)), 0, dptr(c)) == 0
    np.testing.assert_allclose(c, pulay(B), atol=1e-9, rtol=0)


def test_tridiagonal_lowest_eigenpairs_match_numpy():
    """The k lowest eigenpairs of symmetric tridiagonal matrices (the Ritz step of the
    multi-state Lanczos): eigenvalues and eigenvectors (up to sign) against numpy, with a
    close pair of eigenvalues among them."""
    from ansatzevolve_gb300 import dptr, lib
    rng = np.random.default_rng(3)
    for k, nev in [(1, 1), (5, 3), (40, 6), (200, 4)]:
        a = rng.normal(size=k)
        b = rng.normal(size=max(k - 1, 1))[: k - 1] if k > 1 else np.zeros(1)
        if k >= 40:
            a[:2] = [-5.0, -5.0 + 1e-7]
            b[0] = 1e-9
        T = np.diag(a) + (np.diag(b, 1) + np.diag(b, -1) if k > 1 else 0)
        w, V = np.linalg.eigh(T)
        th, Vk = np.zeros(nev), np.zeros(nev * k)
        assert lib().aegpu_host_tridiag_lowest_k(k, nev, dptr(a), dptr(b), dptr(th), dptr(Vk)) == 0
        np.testing.assert_allclose(th, w[:nev], atol=1e-12 * max(1.0, np.abs(w).max()), rtol=0)
        Vk = Vk.reshape(nev, k)
        for j in range(nev):
            np.testing.assert_allclose(np.abs(Vk[j] @ V[:, j]), 1.0, atol=1e-8)
