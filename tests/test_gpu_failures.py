"""Failure paths on the GPU, none of which faults, traps or hangs the device.

- A bounded device wait that gives up reaches the caller as
  HLANC_ERR_DEVICE_TIMEOUT (the reference exits through SAFE_CALL on a CUDA
  error, HLanc.hpp:39-50; this library returns a status instead).  The
  tensor-core basis update waits on its MMAs with an iteration limit;
  opts.wait_limit < 0 makes that wait give up at once.  The CTA that gave up
  still finishes its tile reduction, so the next solve in the same process
  is exact again.
- A NaN in the matrix ends in "not converged" (the reference's return 1,
  HLanc.hpp:1692/1762) or an error, never in a hang.
- A host operator that fails returns HLANC_ERR_CALLBACK through the C ABI;
  the Python mirror re-raises the operator's own exception.
"""
import ctypes as C
import time

import numpy as np
import pytest

from hlanc_gb300 import generators as G

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def H():
    import hlanc_gb300 as H
    from hlanc_gb300 import build
    build.build()
    return H


def _device_out(ncv, n):
    import torch
    return (torch.zeros(ncv, dtype=torch.float64, device="cuda"),
            torch.zeros((ncv, n), dtype=torch.float64, device="cuda"))


def test_device_wait_timeout_reaches_caller(H):
    m = G.laplacian_2d(40, 30)
    op = H.dcsrmv_operator_gpu(m)
    vals, vecs = _device_out(16, m.n)
    good = H.solve_device(op, 6, 16, vals.data_ptr(), vecs.data_ptr(), m.n)
    assert good["rc"] == 0
    ref = vals[:6].cpu().numpy().copy()
    # the first restart's basis update gives up its MMA wait
    with pytest.raises(H.HLancError) as e:
        H.solve_device(op, 6, 16, vals.data_ptr(), vecs.data_ptr(), m.n, wait_limit=-1)
    assert e.value.status == 5          # HLANC_ERR_DEVICE_TIMEOUT
    # the same path with the device restart kernel
    with pytest.raises(H.HLancError) as e:
        H.solve_device(op, 6, 16, vals.data_ptr(), vecs.data_ptr(), m.n, wait_limit=-1,
                       restart_on_device=True)
    assert e.value.status == 5
    # the context is intact and the next solve is bit-identical to the first
    vals.zero_()
    again = H.solve_device(op, 6, 16, vals.data_ptr(), vecs.data_ptr(), m.n)
    assert again["rc"] == 0
    assert np.array_equal(vals[:6].cpu().numpy(), ref)


def test_device_wait_timeout_in_batch_and_server(H):
    mats = [G.laplacian_2d(30, 20), G.banded_random(3000, 4, seed=3, problem=1)]
    ops = [H.dcsrmv_operator_gpu(m) for m in mats]
    outs = [_device_out(12, m.n) for m in mats]
    b = H.Batch(ops, 4, 12, wait_limit=-1)
    with pytest.raises(H.HLancError) as e:
        b.run([v.data_ptr() for v, _ in outs], [x.data_ptr() for _, x in outs])
    assert e.value.status == 5
    b.close()
    srv = H.Server(mem_budget_bytes=1 << 30, max_slots=4)
    bad = srv.submit(ops[0], 4, 12, wait_limit=-1)
    good = srv.submit(ops[1], 4, 12)
    results = {}
    t0 = time.time()
    while len(results) < 2 and time.time() - t0 < 60:
        srv.step()
        for rid in (bad, good):
            if rid not in results:
                r = srv.poll(rid)
                if r is not None:
                    results[rid] = r
    srv.close()
    assert results[bad][0] == 5
    assert results[good][0] == 0


def test_nan_in_matrix_does_not_hang(H):
    m = G.laplacian_2d(20)
    val = m.val.copy()
    rows = np.repeat(np.arange(m.n), np.diff(m.row_ptr))
    hit = np.nonzero((rows == 37) & (m.col == 38))[0][0]
    mirror = np.nonzero((rows == 38) & (m.col == 37))[0][0]
    val[hit] = val[mirror] = np.nan
    bad = G.CSR(m.n, m.ncols, m.row_ptr, m.col, val)
    op = H.dcsrmv_operator_gpu(bad)
    t0 = time.time()
    rc, vals, vecs, st = H.solve(op, 4, 12, max_restarts=50)
    assert rc == 1                      # not converged, like the reference's return 1
    assert time.time() - t0 < 60
    # the FP64 and hybrid CGS kernels and the FP32 SpMV see it the same way
    for kw in (dict(cgs=H.HLANC_CGS_HYBRID), dict(restart_on_device=True)):
        rc, *_ = H.solve(op, 4, 12, max_restarts=20, **kw)
        assert rc == 1
    op32 = H.dcsrmv_operator_gpu(bad, precision=H.HLANC_PREC_FP32_REFINE)
    rc, *_ = H.solve(op32, 4, 12, max_restarts=20, precision=H.HLANC_PREC_FP32_REFINE)
    assert rc == 1


def test_host_operator_failure(H):
    m = G.laplacian_2d(15)
    A = G.to_scipy(m)
    calls = []

    def failing(x, y):
        calls.append(1)
        if len(calls) == 7:
            raise ValueError("operator failed on its 7th call")
        y[:] = A @ x

    values = np.zeros(12)
    vectors = np.zeros((m.n, 12), order="F")
    with pytest.raises(ValueError, match="7th call"):
        H.ds_solver_gpu(m.n, 4, 12, values, vectors, m.n, failing)
    assert len(calls) == 7              # nothing ran after the failure
    # the C ABI itself returns HLANC_ERR_CALLBACK (8)
    seen = []

    def cb(_ctx, xp, yp):
        seen.append(1)
        return 1 if len(seen) == 3 else 0

    fn = H.HOST_OP(cb)
    o, _ = H.opts()
    rc = H.lib().hlanc_solve(0, m.n, 4, 12, values.ctypes.data, vectors.ctypes.data, m.n, None, fn, None,
                             C.byref(o), None)
    assert rc == 8
    assert len(seen) == 3
    # an ordinary solve afterwards still works
    rc, vals, _, _ = H.solve(H.dcsrmv_operator_gpu(m), 4, 12)
    assert rc == 0
