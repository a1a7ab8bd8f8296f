"""The residual verifier that allocates nothing (hlanc_residuals_device_noalloc).

It exists for callers that cannot allocate device memory when they check
Ritz pairs -- a process whose HBM pool is already fully claimed by its own
allocator, or a loop that must not wait on cudaMalloc/cudaFree.  This file
is collected last so that a run stopping at its first failure has already
run every other test.  It calls the entry point through the C ABI twice in a
row, with different inputs, and checks each result against the allocating
entry point (hlanc_residuals_device) to a relative 1e-12: both compute the
same per-row residuals and differ only in the order of the final sums.
"""
import ctypes as C

import numpy as np
import pytest

from hlanc_gb300 import generators as G

pytestmark = pytest.mark.gpu


def _entry(H):
    f = H.lib().hlanc_residuals_device_noalloc
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
    return f


def test_noalloc_residuals_match_the_allocating_entry_point():
    import torch

    import hlanc_gb300 as H
    from hlanc_gb300 import build
    build.build()
    noalloc = _entry(H)
    m = G.laplacian_2d(60, 50)
    op = H.dcsrmv_operator_gpu(m)
    vals = torch.zeros(24, dtype=torch.float64, device="cuda")
    vecs = torch.zeros((24, m.n), dtype=torch.float64, device="cuda")
    st = H.solve_device(op, 8, 24, vals.data_ptr(), vecs.data_ptr(), m.n)
    assert st["rc"] == 0
    # two calls in a row: the converged pairs, then the same vectors with
    # shifted values (residuals of order 1, nothing in common with call 1)
    shifted = vals + 0.25
    for k, lam in ((8, vals), (5, shifted)):
        ref_res, ref_rd = H.residuals_device(op, k, lam.data_ptr(), vecs.data_ptr(), m.n)
        res = np.full(k, np.nan)
        rd = np.full(k, np.nan)
        rc = noalloc(op.handle, k, lam.data_ptr(), vecs.data_ptr(), m.n, res.ctypes.data, rd.ctypes.data)
        assert rc == 0
        assert np.allclose(res, ref_res, rtol=1e-12, atol=0.0), (res, ref_res)
        assert np.allclose(rd, ref_rd, rtol=1e-12, atol=0.0), (rd, ref_rd)
    assert res.min() > 0.1          # the second call did not return the first call's residuals
    # either output may be left out, as with the allocating entry point
    only = np.full(5, np.nan)
    assert noalloc(op.handle, 5, shifted.data_ptr(), vecs.data_ptr(), m.n, only.ctypes.data, None) == 0
    assert np.allclose(only, res, rtol=1e-12, atol=0.0)
    assert noalloc(op.handle, 5, shifted.data_ptr(), vecs.data_ptr(), m.n, None, rd.ctypes.data) == 0
    # more pairs than the fixed scratch holds: a clear error, not a fault
    big = np.zeros(65)
    assert noalloc(op.handle, 65, vals.data_ptr(), vecs.data_ptr(), m.n, big.ctypes.data, big.ctypes.data) == 7
