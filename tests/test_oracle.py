"""The oracle restatement pinned against the reference's own CPU solver
(golden fixtures written by tests/golden/make_golden.py from
ds_solver_mkl + dcsrmv_operator_mkl + dcsr_matrix_t) and against analytic
spectra.  CPU only."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, golden
from hlanc_gb300 import generators as G


def _solve(oracle_mod, m, nev, ncv, seed=0, symmetric=False, **kw):
    x0 = G.start_vector(len(m["row_ptr"]) - 1 if isinstance(m, dict) else m.n, seed)
    if isinstance(m, dict):
        return oracle_mod.solve_csr(m["row_ptr"], m["col"], m["val"], m["ncols"], symmetric, nev, ncv, x0, **kw)
    return oracle_mod.solve_csr(m.row_ptr, m.col, m.val, m.ncols, symmetric, nev, ncv, x0, **kw)


def test_start_vector_bits():
    # SplitMix64 counter generator: pinned first values (seed 0, stream 0)
    v = G.start_vector(4, 0)
    again = G.uniform_pm1(0, 0, 2, offset=2)
    assert np.array_equal(v[2:], again)
    assert np.all((v >= -1) & (v < 1))
    u = G.u64(0, 0, 1)[0]
    assert int(u) == int(G.u64(0, 0, 3)[0])


@pytest.mark.parametrize("case,nev,ncv,gen,sym,rtol", [
    ("c1_laplacian2d_100", 10, 30, lambda: G.laplacian_2d(100), False, 1e-12),
    ("lap3d_12_shift", 20, 60, lambda: G.laplacian_3d(12, shift_seed=1), False, 1e-12),
    ("banded_3000_bw5", 8, 24, lambda: G.banded_random(3000, 5, seed=3, problem=0), False, 1e-12),
    ("chunglu_4096", 16, 48, lambda: G.chung_lu_normalized(4096, seed=2), False, 1e-12),
])
def test_oracle_matches_reference_eigenvalues(oracle_mod, case, nev, ncv, gen, sym, rtol):
    g = golden(f"{case}.npz")
    m = gen()
    rc, vals, vecs, st = _solve(oracle_mod, m, nev, ncv, seed=int(g["seed"]))
    assert rc == 0
    ref = g["values"]
    scale = np.abs(ref).max()
    assert np.abs(vals[:nev] - ref).max() <= rtol * scale
    A = G.to_scipy(m)
    R = A @ vecs[:, :nev] - vecs[:, :nev] * vals[:nev]
    assert np.linalg.norm(R, axis=0).max() <= 1e-10 * scale


def test_oracle_c1_analytic(oracle_mod):
    m = G.laplacian_2d(100)
    rc, vals, _, st = _solve(oracle_mod, m, 10, 30)
    assert rc == 0 and st["nconv"] >= 10
    ana = G.laplacian_2d_eigenvalues(100)[-10:]
    assert np.abs(vals[:10] - ana).max() < 1e-12
    assert np.all(np.diff(vals[:10]) >= 0)      # ascending, largest algebraic


@pytest.mark.parametrize("case,sym", [("simple_pp", False), ("journals_mtx", True)])
def test_oracle_demo_cases_with_vectors(oracle_mod, readers_golden, case, sym):
    tag = "simple" if case == "simple_pp" else "journals"
    m = dict(row_ptr=readers_golden[f"{tag}_row_ptr"], col=readers_golden[f"{tag}_col"],
             val=readers_golden[f"{tag}_val"], ncols=int(readers_golden[f"{tag}_meta"][1]))
    g = golden(f"{case}.npz")
    rc, vals, vecs, _ = _solve(oracle_mod, m, 4, 12, symmetric=sym)
    assert rc == 0
    assert np.abs(vals[:4] - g["values"]).max() <= 1e-12 * np.abs(g["values"]).max()
    dots = np.abs(np.sum(vecs[:, :4] * g["vectors"], axis=0))
    assert np.all(np.abs(dots - 1.0) < 1e-9)


def test_simple_closed_form(oracle_mod):
    # K = min(i,j)+1: lambda_k = 1 / (2 (1 - cos((2k-1) pi / (2n+1))))
    n = 16
    m = G.dense_to_csr(G.simple_dense(n))
    rc, vals, _, _ = _solve(oracle_mod, m, 4, 12)
    k = np.arange(1, n + 1)
    lam = np.sort(1.0 / (2.0 * (1.0 - np.cos((2 * k - 1) * np.pi / (2 * n + 1)))))[-4:]
    assert rc == 0 and np.allclose(vals[:4], lam, rtol=1e-13)


def test_oracle_vectors_odd_grid(oracle_mod):
    g = golden("lap2d_odd_37x23.npz")
    m = G.laplacian_2d(37, 23)
    rc, vals, vecs, _ = _solve(oracle_mod, m, 6, 20, seed=5)
    assert rc == 0
    assert np.abs(vals[:6] - g["values"]).max() < 1e-12
    dots = np.abs(np.sum(vecs[:, :6] * g["vectors"], axis=0))
    assert np.all(np.abs(dots - 1.0) < 1e-8)


def test_spmv_semantics(oracle_mod, readers_golden):
    s = golden("spmv.npz")
    rp, ci, v = readers_golden["journals_row_ptr"], readers_golden["journals_col"], readers_golden["journals_val"]
    n = len(rp) - 1
    y = oracle_mod.spmv(rp, ci, v, n, True, s["x_sym"], kind="mkl")
    assert np.allclose(y, s["y_sym_mkl"], rtol=1e-14, atol=1e-9)
    y2 = oracle_mod.spmv(rp, ci, v, n, True, s["x_sym"], kind="naive")
    assert np.allclose(y2, s["y_sym_naive"], rtol=1e-14, atol=1e-9)
    lap = G.laplacian_2d(7, 5)
    y3 = oracle_mod.spmv(lap.row_ptr, lap.col, lap.val, lap.ncols, False, s["x_gen"])
    assert np.array_equal(y3, s["y_gen"])


def test_readers_bit_exact(oracle_mod, readers_golden, tmp_path):
    g = readers_golden
    i = 0
    while f"c{i}_meta" in g:
        fmt, fn, sym = str(g[f"c{i}_case"]).split("|")
        d = oracle_mod.read_matrix(fmt, os.path.join(GOLDEN, "readers", fn), bool(int(sym)))
        meta = g[f"c{i}_meta"]
        assert [d["nrows"], d["ncols"], d["nnz"], int(d["symmetric"])] == list(meta), (fn, sym)
        assert np.array_equal(d["row_ptr"], g[f"c{i}_row_ptr"])
        assert np.array_equal(d["col"], g[f"c{i}_col"])
        assert np.array_equal(d["val"], g[f"c{i}_val"])
        for wfmt in ("pp", "mm", "bin"):
            key = f"c{i}_save_{wfmt}"
            if key not in g:
                continue
            out = tmp_path / f"c{i}.{wfmt}"
            oracle_mod.save_matrix(wfmt, str(out), d["row_ptr"], d["col"], d["val"], d["ncols"], d["symmetric"])
            assert np.array_equal(np.frombuffer(out.read_bytes(), np.uint8), g[key]), (fn, wfmt)
        i += 1
    assert i >= 8


def test_save_bin_expands_symmetric(oracle_mod, readers_golden, tmp_path):
    g = readers_golden
    out = tmp_path / "j.bin"
    oracle_mod.save_matrix("bin", str(out), g["journals_row_ptr"], g["journals_col"], g["journals_val"],
                           int(g["journals_meta"][1]), True)
    d = oracle_mod.read_matrix("bin", str(out))
    assert np.array_equal(d["row_ptr"], g["journals_bin_row_ptr"])
    assert np.array_equal(d["col"], g["journals_bin_col"])
    assert np.array_equal(d["val"], g["journals_bin_val"])


def test_tridiag_eig(oracle_mod):
    rng = np.random.default_rng(0)
    for n in (1, 2, 5, 30, 60):
        d = rng.standard_normal(n)
        e = rng.standard_normal(max(n - 1, 0))
        rc, w, z = oracle_mod.tridiag_eig(d, e)
        T = np.diag(d) + np.diag(e, 1) + np.diag(e, -1)
        assert rc == 0
        assert np.allclose(w, np.linalg.eigvalsh(T), atol=1e-12)
        assert np.allclose(T @ z, z * w, atol=1e-11)


def test_oracle_rejects_bad_sizes(oracle_mod):
    m = G.laplacian_2d(4)
    x0 = G.start_vector(m.n)
    for nev, ncv in ((4, 4), (3, 17), (0, 5)):
        rc, *_ = oracle_mod.solve_csr(m.row_ptr, m.col, m.val, m.ncols, False, nev, ncv, x0)
        assert rc == 1


@pytest.mark.parametrize("case,nev,ncv,gen", [
    ("lap3d_64_shift", 20, 60, lambda: G.laplacian_3d(64, shift_seed=1)),
    ("chunglu_2e18", 16, 48, lambda: G.chung_lu_normalized(1 << 18, seed=2)),
])
def test_oracle_matches_reference_at_large_n(oracle_mod, case, nev, ncv, gen):
    """The 2^18-row fixtures that pin the GPU's default large-n kernels pin
    the oracle too (all host threads; tens of seconds)."""
    g = golden(f"{case}.npz")
    m = gen()
    rc, vals, _, st = _solve(oracle_mod, m, nev, ncv, seed=int(g["seed"]), threads=os.cpu_count() or 1)
    assert rc == 0
    ref = g["values"]
    assert np.abs(vals[:nev] - ref).max() <= 1e-10 * np.abs(ref).max()


@pytest.mark.parametrize("case,gen", [
    ("lap3d_64_shift", lambda: G.laplacian_3d(64, shift_seed=1)),
    ("chunglu_2e18", lambda: G.chung_lu_normalized(1 << 18, seed=2)),
    ("c2_lap3d_160_shift", lambda: G.laplacian_3d(160, shift_seed=1)),
])
def test_generators_reproduce_fixture_matrices(case, gen):
    """The seeded generators rebuild the matrices the reference solved
    (structure exactly, values to 1e-12 of their checksums)."""
    path = os.path.join(GOLDEN, f"{case}.npz")
    if not os.path.exists(path):
        pytest.skip(f"{case}.npz not generated")
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(GOLDEN, "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    m = gen()
    fp = mg.fingerprint(m.row_ptr, m.col, m.val)
    ref = golden(f"{case}.npz")["fingerprint"]
    assert fp[:4].tolist() == ref[:4].tolist()
    assert np.allclose(fp[4:], ref[4:], rtol=1e-12, atol=0)
