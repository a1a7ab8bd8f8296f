"""GPU parity of ds_solver_gpu / dcsrmv_operator_gpu against the reference's
own CPU solver (golden fixtures from ds_solver_mkl), the oracle, and analytic
spectra.  Tolerances (FP64 mode): eigenvalues within 1e-10 relative of the
reference, residuals ||A v - lambda v|| <= 1e-10 ||A||, eigenvectors equal up
to sign (|<v, v_ref>| within 1e-8 of 1) where the eigenvalue is simple."""
import numpy as np
import pytest

from conftest import golden
from hlanc_gb300 import generators as G

pytestmark = pytest.mark.gpu

EV_RTOL = 1e-10


@pytest.fixture(scope="module")
def H():
    import hlanc_gb300 as H
    from hlanc_gb300 import build
    build.build()
    return H


def _norm_a(m):
    return float(np.abs(G.to_scipy(m)).sum(axis=1).max())


def _check_pairs(m, vals, vecs, k, tol=1e-10):
    A = G.to_scipy(m)
    V = vecs[: m.n, :k]
    R = A @ V - V * vals[:k]
    assert np.linalg.norm(R, axis=0).max() <= tol * _norm_a(m)
    assert np.abs(V.T @ V - np.eye(k)).max() < 1e-10
    assert np.all(np.diff(vals[:k]) >= 0)


@pytest.mark.parametrize("case,gen,nev,ncv", [
    ("c1_laplacian2d_100", lambda: G.laplacian_2d(100), 10, 30),
    ("lap3d_12_shift", lambda: G.laplacian_3d(12, shift_seed=1), 20, 60),
    ("banded_3000_bw5", lambda: G.banded_random(3000, 5, seed=3, problem=0), 8, 24),
    ("chunglu_4096", lambda: G.chung_lu_normalized(4096, seed=2), 16, 48),
])
def test_eigenvalues_match_reference(H, case, gen, nev, ncv):
    g = golden(f"{case}.npz")
    m = gen()
    op = H.dcsrmv_operator_gpu(m)
    rc, vals, vecs, st = H.solve(op, nev, ncv, seed=int(g["seed"]))
    assert rc == 0, st
    assert st["nconv"] >= nev
    ref = g["values"]
    assert np.abs(vals[:nev] - ref).max() <= EV_RTOL * np.abs(ref).max()
    _check_pairs(m, vals, vecs, nev)


def test_c1_analytic(H):
    m = G.laplacian_2d(100)
    op = H.dcsrmv_operator_gpu(m)
    rc, vals, vecs, st = H.solve(op, 10, 30)
    assert rc == 0
    ana = G.laplacian_2d_eigenvalues(100)[-10:]
    assert np.abs(vals[:10] - ana).max() < 1e-12
    _check_pairs(m, vals, vecs, 10)


@pytest.mark.parametrize("case,sym", [("simple_pp", False), ("journals_mtx", True)])
def test_demo_matrices_with_vectors(H, readers_golden, case, sym):
    tag = "simple" if case == "simple_pp" else "journals"
    g = golden(f"{case}.npz")
    mat = H.dcsr_matrix_t.from_arrays(readers_golden[f"{tag}_row_ptr"], readers_golden[f"{tag}_col"],
                                      readers_golden[f"{tag}_val"], int(readers_golden[f"{tag}_meta"][1]), sym)
    n = mat.get_num_rows()
    op = H.dcsrmv_operator_gpu(mat)
    values = np.zeros(12)
    vectors = np.zeros((n, 12), order="F")
    rc = H.ds_solver_gpu(n, 4, 12, values, vectors, n, op)
    assert rc == 0
    ref = g["values"]
    assert np.abs(values[:4] - ref).max() <= EV_RTOL * np.abs(ref).max()
    dots = np.abs(np.sum(vectors[:, :4] * g["vectors"], axis=0))
    assert np.all(np.abs(dots - 1.0) < 1e-8)


def test_function_operator(H):
    # a plain callable as the operator (demo/HLanc_demo.cu:9-18,164)
    K = G.simple_dense(16)

    def op_fun_simple(x, y):
        y[:] = K @ x

    values = np.zeros(12)
    vectors = np.zeros((16, 12), order="F")
    rc = H.ds_solver_gpu(16, 4, 12, values, vectors, 16, op_fun_simple)
    assert rc == 0
    ref = golden("simple_pp.npz")["values"]
    assert np.abs(values[:4] - ref).max() <= EV_RTOL * np.abs(ref).max()
    R = K @ vectors[:, :4] - vectors[:, :4] * values[:4]
    assert np.linalg.norm(R, axis=0).max() < 1e-10 * np.abs(K).sum(axis=1).max()


def test_vectors_odd_grid_and_ldv(H):
    g = golden("lap2d_odd_37x23.npz")
    m = G.laplacian_2d(37, 23)
    op = H.dcsrmv_operator_gpu(m)
    ldv = m.n + 7
    values = np.zeros(20)
    vectors = np.zeros((ldv, 20), order="F")
    vectors[m.n:, :] = 12345.0
    o = H.opts(seed=5)
    rc = H.ds_solver_gpu(m.n, 6, 20, values, vectors, ldv, op, opts_=o)
    assert rc == 0
    assert np.abs(values[:6] - g["values"]).max() < 1e-12 * 8
    dots = np.abs(np.sum(vectors[: m.n, :6] * g["vectors"], axis=0))
    assert np.all(np.abs(dots - 1.0) < 1e-8)
    assert np.all(vectors[m.n:, :] == 12345.0)          # padding rows untouched


def test_matches_oracle_on_same_start(H, oracle_mod):
    m = G.banded_random(1500, 3, seed=11, problem=4)
    x0 = G.start_vector(m.n, 9)
    rc_o, vals_o, vecs_o, _ = oracle_mod.solve_csr(m.row_ptr, m.col, m.val, m.ncols, False, 6, 18, x0)
    op = H.dcsrmv_operator_gpu(m)
    rc, vals, vecs, st = H.solve(op, 6, 18, start=x0)
    assert rc == rc_o == 0
    assert np.abs(vals[:6] - vals_o[:6]).max() <= EV_RTOL * np.abs(vals_o[:6]).max()


@pytest.mark.parametrize("nev,ncv", [(1, 6), (2, 6), (2, 12)])
def test_invariant_subspace_matches_oracle(H, oracle_mod, nev, ncv):
    # two distinct eigenvalues: the Krylov space is exhausted after two steps,
    # the third CGS pass fails and the residual is zeroed (HLanc.hpp:1452-1466);
    # the reference and the oracle return 2.0 (multiplicity 100) nev times
    n = 200
    d = np.array([2.0 if i % 2 else -1.0 for i in range(n)])
    m = G.CSR(n, n, np.arange(n + 1, dtype=np.int32), np.arange(n, dtype=np.int32), d)
    x0 = G.start_vector(n, 3)
    rc_o, vals_o, _, _ = oracle_mod.solve_csr(m.row_ptr, m.col, m.val, n, False, nev, ncv, x0)
    op = H.dcsrmv_operator_gpu(m)
    rc, vals, vecs, st = H.solve(op, nev, ncv, start=x0)
    assert rc == rc_o == 0
    assert np.abs(vals[:nev] - vals_o[:nev]).max() <= EV_RTOL * 2.0
    R = d[:, None] * vecs[:, :nev] - vecs[:, :nev] * vals[:nev]
    assert np.linalg.norm(R, axis=0).max() <= 1e-10 * 2.0


def test_spmv_operator_host_and_device(H, readers_golden):
    import torch
    s = golden("spmv.npz")
    g = readers_golden
    mat = H.dcsr_matrix_t.from_arrays(g["journals_row_ptr"], g["journals_col"], g["journals_val"],
                                      int(g["journals_meta"][1]), True)
    op = H.dcsrmv_operator_gpu(mat)
    y = np.zeros(op.n)
    op(np.ascontiguousarray(s["x_sym"]), y)
    assert np.allclose(y, s["y_sym_mkl"], rtol=1e-13, atol=1e-9)
    xd = torch.from_numpy(s["x_sym"]).cuda()
    yd = torch.zeros_like(xd)
    op(xd, yd)
    torch.cuda.synchronize()
    assert np.allclose(yd.cpu().numpy(), s["y_sym_mkl"], rtol=1e-13, atol=1e-9)
    lap = G.laplacian_2d(7, 5)
    op2 = H.dcsrmv_operator_gpu(lap)
    y2 = np.zeros(lap.n)
    op2(np.ascontiguousarray(s["x_gen"]), y2)
    assert np.allclose(y2, s["y_gen"], rtol=1e-14, atol=1e-14)


def test_spmv_long_rows_and_empty_rows(H, oracle_mod):
    # power-law rows (> 96 entries use the warp path) and empty rows
    rng = np.random.default_rng(5)
    n = 3000
    lens = np.minimum(rng.zipf(1.6, n), 2000)
    lens[::17] = 0
    rp = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    ci = rng.integers(0, n, rp[-1]).astype(np.int32)
    va = rng.standard_normal(rp[-1])
    m = G.CSR(n, n, rp, ci, va)
    op = H.dcsrmv_operator_gpu(m)
    x = rng.standard_normal(n)
    y = np.zeros(n)
    op(x, y)
    ref = oracle_mod.spmv(rp, ci, va, n, False, x, kind="naive")
    assert np.allclose(y, ref, rtol=1e-12, atol=1e-12)


def test_mixed_precision_refined(H):
    g = golden("chunglu_4096.npz")
    m = G.chung_lu_normalized(4096, seed=2)
    op = H.dcsrmv_operator_gpu(m, precision=H.HLANC_PREC_FP32_REFINE)
    rc, vals, vecs, st = H.solve(op, 16, 48, precision=H.HLANC_PREC_FP32_REFINE, seed=int(g["seed"]))
    assert rc == 0, st
    ref = g["values"]
    assert np.abs(vals[:16] - ref).max() <= EV_RTOL * np.abs(ref).max()
    _check_pairs(m, vals, vecs, 16)


def test_tolerance_option(H):
    m = G.laplacian_3d(16, shift_seed=1)
    op = H.dcsrmv_operator_gpu(m)
    rc, vals, vecs, st = H.solve(op, 20, 60, tol=1e-10)
    assert rc == 0
    _check_pairs(m, vals, vecs, 20, tol=1e-9)
    rc2, vals2, _, st2 = H.solve(op, 20, 60)
    assert rc2 == 0
    assert st["spmv_calls"] <= st2["spmv_calls"]
    assert np.abs(vals[:20] - vals2[:20]).max() < 1e-10 * 12


def test_not_converged_returns_1(H):
    m = G.laplacian_2d(60)
    op = H.dcsrmv_operator_gpu(m)
    values = np.zeros(30)
    vectors = np.zeros((m.n, 30), order="F")
    rc = H.ds_solver_gpu(m.n, 10, 30, values, vectors, m.n, op, opts_=H.opts(max_restarts=1))
    assert rc == 1
    assert np.all(values == 0)


def test_invalid_arguments(H):
    m = G.laplacian_2d(8)
    op = H.dcsrmv_operator_gpu(m)
    for nev, ncv in ((4, 4), (3, 65), (0, 4)):
        with pytest.raises(H.HLancError):
            H.ds_solver_gpu(m.n, nev, ncv, np.zeros(70), np.zeros((m.n, 70), order="F"), m.n, op)


def test_graph_and_eager_agree(H):
    m = G.laplacian_2d(50)
    op = H.dcsrmv_operator_gpu(m)
    k0 = H.kernel_launches()
    rc1, v1, _, s1 = H.solve(op, 8, 24, use_graphs=True)
    k1 = H.kernel_launches()
    rc2, v2, _, s2 = H.solve(op, 8, 24, use_graphs=False)
    k2 = H.kernel_launches()
    assert rc1 == rc2 == 0
    assert np.array_equal(v1, v2)                  # same kernels, same order: bit-identical
    assert s1["spmv_calls"] == s2["spmv_calls"]
    # replayed graphs count their kernels like eager launches
    assert k1 - k0 == k2 - k1 > 0, (k1 - k0, k2 - k1)


@pytest.mark.parametrize("gen,nev,ncv", [
    (lambda: G.laplacian_3d(20, shift_seed=1), 20, 60),        # tensor-core basis (ncv <= 64)
    (lambda: G.chung_lu_normalized(4096, seed=2), 16, 48),
    (lambda: G.laplacian_2d(40), 4, 12),
])
def test_basis_tensor_cores_agree_with_fp64(H, gen, nev, ncv):
    # the tensor-core V*Q (FP64-exact integer splitting) and the FP64 kernel
    # give the same pairs to FP64-level accuracy
    m = gen()
    op = H.dcsrmv_operator_gpu(m)
    rc1, v1, x1, s1 = H.solve(op, nev, ncv, tol=1e-10)
    rc2, v2, x2, s2 = H.solve(op, nev, ncv, tol=1e-10, basis_fp64=True)
    assert rc1 == rc2 == 0
    assert np.abs(v1[:nev] - v2[:nev]).max() <= 1e-12 * np.abs(v2[:nev]).max()
    _check_pairs(m, v1, x1, nev)
    assert abs(s1["restarts"] - s2["restarts"]) <= 2


def test_basis_fp64_path_beyond_tensor_core_shape(H):
    # ncv > 64 takes the FP64 kernel under the default setting
    m = G.laplacian_2d(30)
    op = H.dcsrmv_operator_gpu(m)
    rc, vals, vecs, st = H.solve(op, 20, 80, tol=1e-10)
    assert rc == 0
    ref = np.sort(np.linalg.eigvalsh(G.to_scipy(m).toarray()))[-20:]
    assert np.abs(vals[:20] - ref).max() <= EV_RTOL * np.abs(ref).max()
    _check_pairs(m, vals, vecs, 20)


def _dominant(n, k, seed=7):
    # k well-separated dominant eigenvalues (1000, 950, ...) over a bulk in
    # [0, 1), weak nearest-neighbour coupling: converges in the first
    # extension, so no restart runs and both solves share V and Q2 exactly
    rng = np.random.default_rng(seed)
    d = np.concatenate([1000.0 - 50.0 * np.arange(k), rng.random(n - k)])[rng.permutation(n)]
    rp, ci, va = [0], [], []
    for i in range(n):
        for j, x in ((i - 1, 1e-3), (i, d[i]), (i + 1, 1e-3)):
            if 0 <= j < n:
                ci.append(j)
                va.append(x)
        rp.append(len(ci))
    return G.CSR(n, n, np.array(rp, dtype=np.int32), np.array(ci, dtype=np.int32), np.array(va))


@pytest.mark.parametrize("n,nev,ncv", [(3000, 8, 24), (2000, 6, 64), (1000, 4, 12)])
def test_ritz_vectors_tensor_cores_agree_with_fp64(H, n, nev, ncv):
    # All ncv columns of V Q2 from the tensor-core kernel (FP64-exact digit
    # splitting) and from the FP64 kernel, on the same V and Q2: no restart
    # (no basis update) runs in either solve, so only the Ritz kernel differs.
    m = _dominant(n, nev)
    op = H.dcsrmv_operator_gpu(m)
    before = H.variant_counts()
    rc1, v1, x1, s1 = H.solve(op, nev, ncv, tol=1e-10)
    mid = H.variant_counts()
    rc2, v2, x2, s2 = H.solve(op, nev, ncv, tol=1e-10, basis_fp64=True)
    after = H.variant_counts()
    tc = {k: mid[k] - before[k] for k in before}
    fp = {k: after[k] - mid[k] for k in before}
    assert rc1 == rc2 == 0, (s1, s2)
    assert tc["basis_tc"] == tc["basis_fp64"] == fp["basis_tc"] == fp["basis_fp64"] == 0, (tc, fp)
    assert tc["ritz_tc"] == 1 and tc["ritz_fp64"] == 0, tc
    assert fp["ritz_fp64"] == 1 and fp["ritz_tc"] == 0, fp
    assert np.array_equal(v1, v2)
    assert np.abs(x1 - x2).max() <= 1e-13 * np.abs(x2).max()
    _check_pairs(m, v1, x1, nev)
    assert np.abs(x1.T @ x1 - np.eye(ncv)).max() < 1e-12


@pytest.mark.parametrize("case,gen,nev,ncv", [
    ("c1_laplacian2d_100", lambda: G.laplacian_2d(100), 10, 30),
    ("lap3d_12_shift", lambda: G.laplacian_3d(12, shift_seed=1), 20, 60),
    ("banded_3000_bw5", lambda: G.banded_random(3000, 5, seed=3, problem=0), 8, 24),
    ("chunglu_4096", lambda: G.chung_lu_normalized(4096, seed=2), 16, 48),
])
def test_hybrid_cgs_matches_reference(H, case, gen, nev, ncv):
    # the hybrid CGS kernels (part of every column panel as exact fixed-point
    # integer products) forced at sizes where the default keeps FP64
    g = golden(f"{case}.npz")
    m = gen()
    op = H.dcsrmv_operator_gpu(m)
    rc, vals, vecs, st = H.solve(op, nev, ncv, seed=int(g["seed"]), cgs=H.HLANC_CGS_HYBRID)
    assert rc == 0, st
    assert st["nconv"] >= nev
    ref = g["values"]
    assert np.abs(vals[:nev] - ref).max() <= EV_RTOL * np.abs(ref).max()
    _check_pairs(m, vals, vecs, nev)


def _anderson(n, scale, seed=5):
    # random diagonal U(-1, 1) with nearest-neighbour coupling -0.05: the top
    # eigenvectors are localised (entries from ~1 down to ~1e-20)
    rng = np.random.default_rng(seed)
    d = rng.uniform(-1.0, 1.0, n) * scale
    rp, ci, va = [0], [], []
    for i in range(n):
        for j, x in ((i - 1, -0.05 * scale), (i, d[i]), (i + 1, -0.05 * scale)):
            if 0 <= j < n:
                ci.append(j)
                va.append(x)
        rp.append(len(ci))
    return G.CSR(n, n, np.array(rp, dtype=np.int32), np.array(ci, dtype=np.int32), np.array(va))


@pytest.mark.parametrize("scale", [1e-150, 1.0, 1e150])
def test_hybrid_cgs_localised_and_scaled(H, scale):
    # localised basis vectors at extreme operator norms: the fixed-point
    # scales follow w and h, and hybrid and FP64 CGS give the same pairs to
    # FP64-level accuracy.  (At 1e-150 the reference's convergence floor
    # eps * eps^(2/3) is absolute, so the solve stops after one restart and
    # only the agreement of the two kernels is checked.)
    m = _anderson(2000, scale)
    op = H.dcsrmv_operator_gpu(m)
    rc1, v1, x1, s1 = H.solve(op, 6, 24, cgs=H.HLANC_CGS_HYBRID)
    rc2, v2, x2, s2 = H.solve(op, 6, 24, cgs=H.HLANC_CGS_FP64)
    assert rc1 == rc2 == 0
    assert np.abs(v1[:6] - v2[:6]).max() <= 1e-12 * np.abs(v2[:6]).max()
    if scale >= 1.0:
        _check_pairs(m, v1, x1, 6)
        ref = np.linalg.eigvalsh(G.to_scipy(m).toarray())[-6:]
        assert np.abs(v1[:6] - ref).max() <= EV_RTOL * np.abs(ref).max()


def test_hybrid_cgs_default_on_large_problem(H):
    # 2^18 rows: the default picks the hybrid kernels; same pairs as FP64
    m = G.chung_lu_normalized(2 ** 18, seed=2)
    op = H.dcsrmv_operator_gpu(m)
    rc1, v1, x1, s1 = H.solve(op, 8, 24, tol=1e-10)
    rc2, v2, x2, s2 = H.solve(op, 8, 24, tol=1e-10, cgs=H.HLANC_CGS_FP64)
    assert rc1 == rc2 == 0
    assert np.abs(v1[:8] - v2[:8]).max() <= 1e-12 * np.abs(v2[:8]).max()
    _check_pairs(m, v1, x1, 8)


def test_hybrid_cgs_host_operator_and_mixed_precision(H):
    # forced hybrid CGS where w arrives from a host callback, and in the
    # FP32 phase + FP64 refinement of a mixed-precision solve (the shifted
    # 3-D Laplacian has simple eigenvalues; single-vector Lanczos returns
    # one copy of a multiple one)
    m = G.laplacian_3d(10, shift_seed=1)
    A = G.to_scipy(m)

    def op(x, y):
        y[:] = A @ x

    o = H.opts(cgs=H.HLANC_CGS_HYBRID, tol=1e-10)        # (opts, buffers it keeps alive)
    values = np.zeros(16)
    vectors = np.zeros((m.n, 16), order="F")
    rc = H.ds_solver_gpu(m.n, 4, 16, values, vectors, m.n, op, opts_=o)
    assert rc == 0
    ref = np.sort(np.linalg.eigvalsh(A.toarray()))[-4:]
    assert np.abs(values[:4] - ref).max() <= EV_RTOL * np.abs(ref).max()
    _check_pairs(m, values, vectors, 4)

    g = golden("chunglu_4096.npz")
    m2 = G.chung_lu_normalized(4096, seed=2)
    op2 = H.dcsrmv_operator_gpu(m2, precision=H.HLANC_PREC_FP32_REFINE)
    rc, vals, vecs, st = H.solve(op2, 16, 48, precision=H.HLANC_PREC_FP32_REFINE, seed=int(g["seed"]),
                                 cgs=H.HLANC_CGS_HYBRID)
    assert rc == 0, st
    assert np.abs(vals[:16] - g["values"]).max() <= EV_RTOL * np.abs(g["values"]).max()
    _check_pairs(m2, vals, vecs, 16)


def test_largest_basis(H):
    # ncv = HLANC_MAX_NCV with nev 40: the adjusted nev grows past 64 (up to
    # half of np is added), so the restart takes the wide basis kernel; the
    # hybrid CGS kernels carry up to 128 columns (the update's integer
    # accumulators at their Cauchy-Schwarz bound)
    m = G.laplacian_3d(20, shift_seed=1)
    op = H.dcsrmv_operator_gpu(m)
    ncv = H.HLANC_MAX_NCV
    ref = np.sort(np.linalg.eigvalsh(G.to_scipy(m).toarray()))[-40:]
    rc1, v1, x1, s1 = H.solve(op, 40, ncv, tol=1e-10, cgs=H.HLANC_CGS_HYBRID)
    rc2, v2, x2, s2 = H.solve(op, 40, ncv, tol=1e-10, cgs=H.HLANC_CGS_FP64)
    assert rc1 == rc2 == 0
    for v, x in ((v1, x1), (v2, x2)):
        assert np.abs(v[:40] - ref).max() <= EV_RTOL * np.abs(ref).max()
        _check_pairs(m, v, x, 40)
    assert np.abs(v1[:40] - v2[:40]).max() <= 1e-12 * np.abs(v2[:40]).max()


def test_largest_basis_device_restart(H):
    # the same envelope with the restart math in device kernels
    m = G.laplacian_3d(20, shift_seed=1)
    op = H.dcsrmv_operator_gpu(m)
    ref = np.sort(np.linalg.eigvalsh(G.to_scipy(m).toarray()))[-40:]
    rc, v, x, st = H.solve(op, 40, H.HLANC_MAX_NCV, tol=1e-10, restart_on_device=True)
    assert rc == 0, st
    assert np.abs(v[:40] - ref).max() <= EV_RTOL * np.abs(ref).max()
    _check_pairs(m, v, x, 40)


def test_largest_nev_tensor_core_basis(H):
    # nev = HLANC_MAX_NEV with ncv = 64: the tensor-core basis update at its
    # widest (nev + 1 = 64 outputs).  With np = 1 a restart adds one Lanczos
    # step, so the spectrum is chosen to converge fast: 63 large, separated
    # eigenvalues above a tight cluster near zero, weakly coupled.
    n = 400
    rng = np.random.default_rng(21)
    d = np.concatenate([100.0 + 3.0 * np.arange(63), 1e-3 * rng.random(n - 63)])
    d = d[rng.permutation(n)]
    rp, ci, va = [0], [], []
    for i in range(n):
        for j, x in ((i - 1, 1e-3), (i, d[i]), (i + 1, 1e-3)):
            if 0 <= j < n:
                ci.append(j)
                va.append(x)
        rp.append(len(ci))
    m = G.CSR(n, n, np.array(rp, dtype=np.int32), np.array(ci, dtype=np.int32), np.array(va))
    op = H.dcsrmv_operator_gpu(m)
    nev = H.HLANC_MAX_NEV
    ref = np.sort(np.linalg.eigvalsh(G.to_scipy(m).toarray()))[-nev:]
    before = H.variant_counts()
    rc, v, x, st = H.solve(op, nev, 64, tol=1e-10)
    used = {k: c - before[k] for k, c in H.variant_counts().items()}
    assert rc == 0, st
    assert np.abs(v[:nev] - ref).max() <= EV_RTOL * np.abs(ref).max()
    _check_pairs(m, v, x, nev)
    # the restarts took the tensor-core update at 64 outputs, never the FP64 kernel
    assert st["restarts"] > 0 and used["basis_tc"] > 0 and used["basis_fp64"] == 0, used


def test_cgs_kernels_alone(H):
    # hlanc_diag_cgs: both CGS kernels run on a synthetic basis and report
    # positive times; the hybrid one is not slower than FP64 at this size
    fp = H.cgs_kernel_ms(1 << 20, 24, H.HLANC_CGS_FP64, reps=3)
    hy = H.cgs_kernel_ms(1 << 20, 24, H.HLANC_CGS_HYBRID, reps=3)
    for r in (fp, hy):
        assert all(0.0 < v < 1000.0 for v in r.values()), r
    assert hy["proj"] <= 1.1 * fp["proj"]


def test_native_library_loaded(H):
    import os
    with open("/proc/self/maps") as f:
        maps = f.read()
    assert os.path.basename(H.LIB_PATH) in maps
    assert H.kernel_launches() > 0


def test_host_outputs_pinned_and_pageable_agree(H):
    # Outputs above 64 MB: a pinned host buffer (mapped into the device's
    # address space) is written by the library's copy kernel, 16-byte and
    # 8-byte forms (even and odd ldv); a pageable one is page-locked and
    # copied by DMA.  Same pairs, bit for bit.
    import torch
    m = G.laplacian_3d(60, shift_seed=1)          # 216,000 rows; 40 columns = 69 MB
    op = H.dcsrmv_operator_gpu(m)
    nev, ncv = 10, 40
    out = {}
    for kind, ldv in (("pageable", m.n), ("pinned", m.n), ("pinned", m.n + 1)):
        values = np.zeros(ncv)
        if kind == "pinned":
            vectors = torch.zeros(ldv * ncv, dtype=torch.float64, pin_memory=True).numpy()
        else:
            vectors = np.zeros(ldv * ncv)
        vectors[:] = 7.0
        st = {}
        rc = H.ds_solver_gpu(m.n, nev, ncv, values, vectors, ldv, op, opts_=H.opts(tol=1e-10), stats=st)
        assert rc == 0, st
        X = vectors.reshape(ncv, ldv).T
        if ldv > m.n:
            assert np.all(X[m.n:, :] == 7.0)       # padding rows untouched
        out[(kind, ldv)] = (values.copy(), np.ascontiguousarray(X[: m.n, :]))
    ref_v, ref_x = out[("pageable", m.n)]
    for key, (v, x) in out.items():
        assert np.array_equal(v, ref_v), key
        assert np.array_equal(x, ref_x), key
    _check_pairs(m, ref_v, ref_x, nev)
