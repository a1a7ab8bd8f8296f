"""GPU parity at the sizes where the default kernels change: launches over
>= 2^18 rows take the hybrid (FP64 + fixed-point) CGS projection, every
solve takes the FP32-copy CGS update and (ncv <= 64) the tensor-core basis
update.  The anchors are the reference's own CPU solver (ds_solver_mkl +
dcsrmv_operator_mkl, HLanc.hpp:1650-1861) run on the same matrices from the
same start vector (tests/golden/*.npz, written by make_golden.py --large /
--full).

Tolerances: eigenvalues within 1e-10 relative of the reference (FP64 mode
and the mixed FP32-SpMV + FP64-refinement mode alike, since the refinement
runs to the same tolerance), residuals ||A v - lambda v|| <= 1e-10 ||A||_inf.
Each test first checks the regenerated matrix against the fixture's
fingerprint, so a generator change cannot pass for a solver change.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN, golden
from hlanc_gb300 import generators as G

pytestmark = pytest.mark.gpu

EV_RTOL = 1e-10

CASES = [
    ("lap3d_64_shift", lambda: G.laplacian_3d(64, shift_seed=1), 20, 60),
    ("chunglu_2e18", lambda: G.chung_lu_normalized(1 << 18, seed=2), 16, 48),
]
FULL = [
    ("c2_lap3d_160_shift", lambda: G.laplacian_3d(160, shift_seed=1), 20, 60),
    ("c3_chunglu_2e22", lambda: G.chung_lu_normalized(1 << 22, seed=2), 16, 48),
]


@pytest.fixture(scope="module")
def H():
    import hlanc_gb300 as H
    from hlanc_gb300 import build
    build.build()
    return H


def _fingerprint(m):
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(GOLDEN, "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    return mg.fingerprint(m.row_ptr, m.col, m.val)


def _check_matrix(g, m):
    fp = _fingerprint(m)
    ref = g["fingerprint"]
    assert fp[:2].tolist() == ref[:2].tolist()           # n, nnz
    assert np.allclose(fp[2:], ref[2:], rtol=1e-12, atol=0), (fp, ref)


def _norm_a(m):
    return float(np.abs(G.to_scipy(m)).sum(axis=1).max())


def _solve_and_check(H, g, m, nev, ncv, prec):
    import torch
    op = H.dcsrmv_operator_gpu(m, precision=prec)
    before = H.variant_counts()
    vals = torch.zeros(ncv, dtype=torch.float64, device="cuda")
    vecs = torch.zeros((ncv, m.n), dtype=torch.float64, device="cuda")
    st = H.solve_device(op, nev, ncv, vals.data_ptr(), vecs.data_ptr(), m.n, precision=prec,
                        seed=int(g["seed"]))
    after = H.variant_counts()
    assert st["rc"] == 0 and st["nconv"] >= nev, st
    got = vals[:nev].cpu().numpy()
    ref = g["values"]
    err = np.abs(got - ref).max() / np.abs(ref).max()
    assert err <= EV_RTOL, (err, got, ref)
    res, _ = H.residuals_device(op, nev, vals.data_ptr(), vecs.data_ptr(), m.n)
    assert res.max() <= 1e-10 * _norm_a(m), res
    return st, {k: after[k] - before[k] for k in after}


@pytest.mark.parametrize("case,gen,nev,ncv", CASES)
@pytest.mark.parametrize("mixed", [False, True])
def test_default_large_path_matches_reference(H, case, gen, nev, ncv, mixed):
    g = golden(f"{case}.npz")
    m = gen()
    _check_matrix(g, m)
    prec = H.HLANC_PREC_FP32_REFINE if mixed else H.HLANC_PREC_FP64
    st, used = _solve_and_check(H, g, m, nev, ncv, prec)
    # the default kernels at this size: hybrid projection, FP32-copy update,
    # tensor-core basis update; none of the all-FP64 CGS kernels
    assert used["proj_hybrid"] > 0 and used["proj_fp64"] == 0, used
    assert used["apply_shadow"] > 0 and used["apply_fp64"] == 0, used
    assert used["basis_tc"] > 0 and used["basis_fp64"] == 0, used


@pytest.mark.parametrize("case,gen,nev,ncv", CASES)
def test_spmv_units_tuned_from_row_histogram(H, case, gen, nev, ncv):
    """Uneven rows (the power-law graph) are tuned on the device; uniform
    short rows (the Laplacian) keep the default units untimed."""
    m = gen()
    t = H.dcsrmv_operator_gpu(m).tuning()
    if case.startswith("chunglu"):
        assert t["us_default"] > 0 and 0 < t["us_chosen"] <= t["us_default"], t
    else:
        assert t["us_default"] == 0 and t["rows_per_unit"] == 1024, t


def _with_empty_rows(m, every=7):
    """The matrix with every `every`-th row emptied (empty rows and uneven
    lengths in the same sliced-ELL windows)."""
    A = G.to_scipy(m).tolil()
    for r in range(0, m.n, every):
        A.rows[r] = []
        A.data[r] = []
    A = A.tocsr()
    return G.CSR(m.n, m.ncols, A.indptr.astype(np.int32), A.indices.astype(np.int32), A.data.astype(np.float64))


@pytest.mark.parametrize("gen", [lambda: G.chung_lu_normalized(1 << 18, seed=2),
                                 lambda: G.banded_random(1 << 17, 12, seed=3, problem=9),
                                 lambda: _with_empty_rows(G.chung_lu_normalized(1 << 17, seed=5))])
def test_tuned_spmv_layout_matches_scipy(H, gen):
    """Whichever layout the tuner keeps for an uneven matrix (row-class units
    or the sliced-ELL copy), y = A x agrees with scipy's product to FP64
    rounding (|y - Ax| <= 1e-13 |A||x| per row), and the FP32 SpMV within
    the worst-case FP32 bound (row length + 2) 2^-24 |A||x|."""
    import torch
    m = gen()
    A = G.to_scipy(m)
    x = np.random.default_rng(1).uniform(-1.0, 1.0, m.n)
    ref = A @ x
    scale = abs(A) @ np.abs(x)
    op = H.dcsrmv_operator_gpu(m, precision=H.HLANC_PREC_FP32_REFINE)
    t = op.tuning()
    assert t["us_chosen"] > 0, t
    y = np.zeros(m.n)
    op(x, y)
    assert np.all(np.abs(y - ref) <= 1e-13 * scale), (t, float(np.max(np.abs(y - ref) / scale)))
    xd = torch.tensor(x, dtype=torch.float32, device="cuda")
    yd = torch.zeros(m.n, dtype=torch.float32, device="cuda")
    H.lib().hlanc_csr_spmv_f32_async(op.handle, xd.data_ptr(), yd.data_ptr(), None)
    torch.cuda.synchronize()
    y32 = yd.cpu().numpy().astype(np.float64)
    rl = np.diff(A.indptr).astype(np.float64)
    assert np.all(np.abs(y32 - ref) <= (rl + 2.0) * 2.0 ** -24 * scale + 1e-30), t


@pytest.mark.parametrize("case,gen,nev,ncv", CASES[:1])
def test_all_fp64_kernels_match_reference_at_large_n(H, case, gen, nev, ncv):
    g = golden(f"{case}.npz")
    m = gen()
    op = H.dcsrmv_operator_gpu(m)
    before = H.variant_counts()
    rc, vals, vecs, st = H.solve(op, nev, ncv, cgs=H.HLANC_CGS_FP64, basis_fp64=True)
    after = H.variant_counts()
    assert rc == 0
    ref = g["values"]
    assert np.abs(vals[:nev] - ref).max() <= EV_RTOL * np.abs(ref).max()
    used = {k: after[k] - before[k] for k in after}
    assert used["proj_hybrid"] == 0 and used["apply_shadow"] == 0 and used["basis_tc"] == 0, used


@pytest.mark.parametrize("case,gen,nev,ncv", FULL)
def test_full_size_workloads_match_reference(H, case, gen, nev, ncv):
    """The two single-solve workloads at full size (n = 4,096,000 and 2^22)."""
    if not os.path.exists(os.path.join(GOLDEN, f"{case}.npz")):
        pytest.skip(f"{case}.npz not generated")
    g = golden(f"{case}.npz")
    m = gen()
    _check_matrix(g, m)
    _solve_and_check(H, g, m, nev, ncv, H.HLANC_PREC_FP64)
    if case.startswith("c3"):      # the power-law workload's own precision mode too
        _solve_and_check(H, g, m, nev, ncv, H.HLANC_PREC_FP32_REFINE)
