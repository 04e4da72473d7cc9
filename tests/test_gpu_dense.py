"""The FP64 Gram kernel of the Hessian and properties passes (csrc/dense.cu) on its own:
upper triangle of alpha * A^H B against numpy at sizes that cut panels, micro-tiles and
row slabs unevenly, real and complex, with padded column strides; and bit-identical
repeats (fixed reduction order)."""
import numpy as np
import pytest

import ansatzevolve_gb300 as ae

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("W,V,nrows", [(1, 1, 5), (1, 3, 1000), (1, 64, 4097), (1, 65, 777), (1, 100, 13340),
                                       (1, 200, 33), (2, 1, 17), (2, 7, 3001), (2, 130, 999)])
def test_gram_upper_matches_numpy(W, V, nrows):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(V * 1000 + nrows)
    lda = nrows * W + 8
    A = rng.normal(size=(V, lda))
    B = rng.normal(size=(V, lda))
    dev = torch.device("cuda")
    Ad, Bd = torch.tensor(A, device=dev), torch.tensor(B, device=dev)
    stream = torch.cuda.current_stream().cuda_stream
    outs = []
    for _ in range(2):
        Cre = torch.full((V, V), np.nan, dtype=torch.float64, device=dev)
        Cim = torch.full((V, V), np.nan, dtype=torch.float64, device=dev)
        rc = ae.lib().aegpu_gram_upper_dev(Ad.data_ptr(), lda, Bd.data_ptr(), lda, nrows, W, V, 2.0, Cre.data_ptr(),
                                           Cim.data_ptr(), V, stream)
        assert rc == 0
        torch.cuda.synchronize()
        # column-major (i + j * V) -> the tensor's [j, i]
        outs.append((Cre.cpu().numpy().T.copy(), Cim.cpu().numpy().T.copy()))
    a = A[:, :nrows * W]
    b = B[:, :nrows * W]
    if W == 1:
        want_re, want_im = 2.0 * a @ b.T, None
    else:
        za = a[:, 0::2] + 1j * a[:, 1::2]
        zb = b[:, 0::2] + 1j * b[:, 1::2]
        z = 2.0 * za.conj() @ zb.T
        want_re, want_im = z.real, z.imag
    iu = np.triu_indices(V)
    il = np.tril_indices(V, -1)
    tol = 1e-13 * 2.0 * np.sqrt(nrows * W) * 4
    np.testing.assert_allclose(outs[0][0][iu], want_re[iu], rtol=0, atol=tol)
    assert np.all(np.isnan(outs[0][0][il]))  # below the diagonal untouched
    if W == 2:
        np.testing.assert_allclose(outs[0][1][iu], want_im[iu], rtol=0, atol=tol)
    np.testing.assert_array_equal(outs[0][0][iu], outs[1][0][iu])
