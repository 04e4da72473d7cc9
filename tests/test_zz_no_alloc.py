"""The allocation-free H * x entry point (aegpu_csr_energy_noalloc).

It serves callers that cannot allocate device memory (allocator callbacks, host
frameworks that own the device budget): it keeps its scratch in a fixed device array
instead of cudaMalloc.  This test calls it through the C ABI and checks y = H x and
<x|H x> against the engine's own entry point (aegpu_apply_dev, which uses scratch the
engine allocated) and against an independent host product of the same CSR arrays, on
two calls in a row, and that an input over the fixed limit and an in-place call
(x == y) are rejected.  Collected last so that a run stopping at the first failure has already run
every other test; it also passes on its own in a fresh process.
"""
import numpy as np
import pytest

import ansatzevolve_gb300 as ae
from tests.fixtures import oracle_synthetic, synthetic_problem

pytestmark = pytest.mark.gpu


def test_noalloc_energy_matches_engine_entry_point():
    torch = pytest.importorskip("torch")
    L = ae.lib()
    pb = synthetic_problem(8, 4, 4, 2, 0)
    o = oracle_synthetic(pb, csr=True)
    rp, col, val = o.csr()
    D = int(o.D)
    eng = ae.Engine(16, ae.BASIS_SZ, 8, 4, 4, np.asarray(pb["ops_1b"]) - 1)
    eng.set_ham_csr(rp, col, val)
    dev = torch.device("cuda")
    rp_d = torch.tensor(rp, dtype=torch.int64, device=dev)
    col_d = torch.tensor(col, dtype=torch.int32, device=dev)
    val_d = torch.tensor(val, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream().cuda_stream
    rng = np.random.default_rng(5)
    for call in range(2):
        x = torch.tensor(rng.normal(size=D), dtype=torch.float64, device=dev)
        y_ref = torch.zeros(D, dtype=torch.float64, device=dev)
        e_ref = torch.zeros(1, dtype=torch.float64, device=dev)
        eng.apply_dev(x.data_ptr(), y_ref.data_ptr(), e_ref.data_ptr(), stream)
        y = torch.full((D,), np.nan, dtype=torch.float64, device=dev)
        e = torch.full((1,), np.nan, dtype=torch.float64, device=dev)
        rc = L.aegpu_csr_energy_noalloc(D, rp_d.data_ptr(), col_d.data_ptr(), val_d.data_ptr(), x.data_ptr(),
                                        y.data_ptr(), e.data_ptr(), stream)
        assert rc == 0, call
        torch.cuda.synchronize()
        np.testing.assert_allclose(y.cpu().numpy(), y_ref.cpu().numpy(), atol=1e-12, rtol=0)
        assert abs(float(e.item()) - float(e_ref.item())) < 1e-10
        # independent host product of the caller's CSR arrays: y_r = sum_k val_k x[col_k]
        xh = x.cpu().numpy()
        rows = np.repeat(np.arange(D), np.diff(rp))
        y_host = np.bincount(rows, weights=val * xh[col], minlength=D)
        np.testing.assert_allclose(y.cpu().numpy(), y_host, atol=1e-12, rtol=0)
        assert abs(float(e.item()) - float(xh @ y_host)) < 1e-10
    # over the fixed limit: rejected before any launch
    too_big = 4194304 + 1
    rc = L.aegpu_csr_energy_noalloc(too_big, rp_d.data_ptr(), col_d.data_ptr(), val_d.data_ptr(), x.data_ptr(),
                                    y.data_ptr(), e.data_ptr(), stream)
    assert rc == 6
    # the product is not in place: x == y is refused before any launch
    rc = L.aegpu_csr_energy_noalloc(D, rp_d.data_ptr(), col_d.data_ptr(), val_d.data_ptr(), x.data_ptr(),
                                    x.data_ptr(), e.data_ptr(), stream)
    assert rc == 1
    eng.close()
