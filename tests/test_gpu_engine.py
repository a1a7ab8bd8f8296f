"""GPU tests of the engine beyond a single plain solve: batched solves,
continuous-batching serving (each result equal alone and in the mix), the
device-restart path, launch profiling, the residual verifier and the C++
drop-in header end to end.  Tolerances as in test_gpu_solver.py."""
import os
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, ROOT, golden
from hlanc_gb300 import generators as G

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def H():
    import hlanc_gb300 as H
    from hlanc_gb300 import build
    build.build()
    return H


@pytest.fixture(scope="module")
def torch():
    import torch
    return torch


def _norm_a(m):
    return float(np.abs(G.to_scipy(m)).sum(axis=1).max())


def test_device_restart_path_agrees(H):
    m = G.laplacian_2d(40)
    op = H.dcsrmv_operator_gpu(m)
    rc1, v1, x1, s1 = H.solve(op, 6, 18)
    rc2, v2, x2, s2 = H.solve(op, 6, 18, restart_on_device=True)
    assert rc1 == rc2 == 0
    assert np.abs(v1[:6] - v2[:6]).max() < 1e-12 * 8
    R = G.to_scipy(m) @ x2[:, :6] - x2[:, :6] * v2[:6]
    assert np.linalg.norm(R, axis=0).max() < 1e-10 * 8


def test_profile_classes(H):
    m = G.laplacian_3d(20, shift_seed=1)
    op = H.dcsrmv_operator_gpu(m)
    # per-phase launches
    rc, vals, _, st = H.solve(op, 10, 30, tol=1e-10, profile=True, cycle=H.HLANC_CYCLE_OFF)
    assert rc == 0
    p = H.last_profile()
    assert p["spmv"]["launches"] >= st["spmv_calls"]
    assert p["cgs_proj"]["launches"] > 0 and p["cgs_proj"]["ms"] > 0
    assert p["cgs_apply"]["bytes"] > 0 and p["basis"]["launches"] > 0
    assert p["host_restart"]["launches"] == st["restarts"]
    assert p["cycle"]["launches"] == 0
    # the default on a problem this small: one launch per extension
    rc2, vals2, _, st2 = H.solve(op, 10, 30, tol=1e-10, profile=True)
    assert rc2 == 0
    p = H.last_profile()
    assert p["cycle"]["launches"] == st2["restarts"] and p["cycle"]["bytes"] > 0
    assert p["spmv"]["launches"] == 0 and p["cgs_proj"]["launches"] == 0
    assert np.abs(vals2[:10] - vals[:10]).max() <= 1e-10 * np.abs(vals[:10]).max()


def test_residual_verifier(H, torch):
    m = G.laplacian_2d(30)
    op = H.dcsrmv_operator_gpu(m)
    vals = torch.zeros(15, dtype=torch.float64, device="cuda")
    vecs = torch.zeros((15, m.n), dtype=torch.float64, device="cuda")
    st = H.solve_device(op, 5, 15, vals.data_ptr(), vecs.data_ptr(), m.n)
    assert st["rc"] == 0
    res, rd = H.residuals_device(op, 5, vals.data_ptr(), vecs.data_ptr(), m.n)
    V = vecs.cpu().numpy()[:5].T
    lam = vals.cpu().numpy()[:5]
    R = G.to_scipy(m) @ V - V * lam
    assert np.allclose(res, np.linalg.norm(R, axis=0), rtol=1e-6, atol=1e-14)
    assert res.max() < 1e-10 * 8 and rd.max() < 1e-9


def _batch_mats(count, seed=3, n_lo=500, n_hi=4000):
    ns, bws = G.batched_problem_sizes(count, n_lo, n_hi, 2, 8, seed=seed)
    return [G.banded_random(int(n), int(b), seed=seed, problem=i) for i, (n, b) in enumerate(zip(ns, bws))]


def test_batch_matches_solo(H, torch):
    mats = _batch_mats(12)
    ops = [H.dcsrmv_operator_gpu(m) for m in mats]
    b = H.Batch(ops, 4, 12)
    vals = [torch.zeros(12, dtype=torch.float64, device="cuda") for _ in mats]
    vecs = [torch.zeros((12, m.n), dtype=torch.float64, device="cuda") for m in mats]
    status, st = b.run([v.data_ptr() for v in vals], [x.data_ptr() for x in vecs])
    assert np.all(status == 0), status
    for m, op, v, x in zip(mats, ops, vals, vecs):
        rc, sv, _, _ = H.solve(op, 4, 12)
        assert rc == 0
        got = v.cpu().numpy()[:4]
        assert np.abs(got - sv[:4]).max() <= 1e-10 * np.abs(sv[:4]).max()
        X = x.cpu().numpy()[:4].T
        R = G.to_scipy(m) @ X - X * got
        assert np.linalg.norm(R, axis=0).max() <= 1e-10 * _norm_a(m)


def test_batch_hybrid_cgs_matches_solo(H, torch):
    # forced hybrid CGS in a batched launch (descriptors from the launch
    # tables, one tile table over all problems) against FP64 solo solves
    mats = _batch_mats(8, seed=11)
    ops = [H.dcsrmv_operator_gpu(m) for m in mats]
    b = H.Batch(ops, 4, 12, cgs=H.HLANC_CGS_HYBRID)
    vals = [torch.zeros(12, dtype=torch.float64, device="cuda") for _ in mats]
    vecs = [torch.zeros((12, m.n), dtype=torch.float64, device="cuda") for m in mats]
    status, st = b.run([v.data_ptr() for v in vals], [x.data_ptr() for x in vecs])
    assert np.all(status == 0), status
    for m, op, v, x in zip(mats, ops, vals, vecs):
        rc, sv, _, _ = H.solve(op, 4, 12, cgs=H.HLANC_CGS_FP64)
        assert rc == 0
        got = v.cpu().numpy()[:4]
        assert np.abs(got - sv[:4]).max() <= 1e-10 * np.abs(sv[:4]).max()
        X = x.cpu().numpy()[:4].T
        R = G.to_scipy(m) @ X - X * got
        assert np.linalg.norm(R, axis=0).max() <= 1e-10 * _norm_a(m)


def test_batch_mixed_basis_widths(H, torch):
    # one problem with ncv = 100 (its adjusted nev passes 64, so the whole
    # launch takes the wide basis kernel) batched with small ones; each
    # problem keeps its own nev inside that kernel
    mats = [G.laplacian_3d(12, shift_seed=1)] + _batch_mats(2, seed=13)
    nevs = [30, 4, 4]
    ncvs = [100, 12, 12]
    ops = [H.dcsrmv_operator_gpu(m) for m in mats]
    b = H.Batch(ops, nevs, ncvs, tol=1e-10)
    vals = [torch.zeros(c, dtype=torch.float64, device="cuda") for c in ncvs]
    vecs = [torch.zeros((c, m.n), dtype=torch.float64, device="cuda") for c, m in zip(ncvs, mats)]
    status, st = b.run([v.data_ptr() for v in vals], [x.data_ptr() for x in vecs])
    assert np.all(status == 0), status
    for m, op, v, x, k, c in zip(mats, ops, vals, vecs, nevs, ncvs):
        ref = np.sort(np.linalg.eigvalsh(G.to_scipy(m).toarray()))[-k:]
        got = v.cpu().numpy()[:k]
        assert np.abs(got - ref).max() <= 1e-10 * np.abs(ref).max()
        X = x.cpu().numpy()[:k].T
        R = G.to_scipy(m) @ X - X * got
        assert np.linalg.norm(R, axis=0).max() <= 1e-10 * _norm_a(m)


def test_batch_mixed_precision(H, torch):
    mats = _batch_mats(6, seed=5)
    ops = [H.dcsrmv_operator_gpu(m, precision=H.HLANC_PREC_FP32_REFINE) for m in mats]
    b = H.Batch(ops, 4, 12, precision=H.HLANC_PREC_FP32_REFINE)
    vals = [torch.zeros(12, dtype=torch.float64, device="cuda") for _ in mats]
    vecs = [torch.zeros((12, m.n), dtype=torch.float64, device="cuda") for m in mats]
    status, st = b.run([v.data_ptr() for v in vals], [x.data_ptr() for x in vecs])
    assert np.all(status == 0), status
    for m, v, x in zip(mats, vals, vecs):
        ref = np.sort(np.linalg.eigvalsh(G.to_scipy(m).toarray()))[-4:]
        got = v.cpu().numpy()[:4]
        assert np.abs(got - ref).max() <= 1e-10 * np.abs(ref).max()
        X = x.cpu().numpy()[:4].T
        R = G.to_scipy(m) @ X - X * got
        assert np.linalg.norm(R, axis=0).max() <= 1e-10 * _norm_a(m)


def test_server_continuous_batching_same_alone_and_in_mix(H):
    mats = _batch_mats(10, seed=7, n_lo=800, n_hi=6000)
    ops = [H.dcsrmv_operator_gpu(m) for m in mats]
    solo = [H.solve(op, 4, 12) for op in ops]
    srv = H.Server(mem_budget_bytes=64 << 20, max_slots=4)
    ids = []
    done = {}
    # staggered arrivals: two requests per tick while earlier ones run
    pending = list(range(len(ops)))
    ticks = 0
    while len(done) < len(ops):
        for _ in range(2):
            if pending:
                i = pending.pop(0)
                ids.append((i, srv.submit(ops[i], 4, 12)))
        active, waiting = srv.step()
        assert active <= 4
        ticks += 1
        for i, rid in ids:
            if i not in done:
                r = srv.poll(rid)
                if r is not None:
                    done[i] = r
        assert ticks < 5000
    for i, (status, vals, vecs, st) in done.items():
        assert status == 0
        rc, sv, sx, _ = solo[i]
        assert np.abs(vals[:4] - sv[:4]).max() <= 1e-12 * np.abs(sv[:4]).max()
        dots = np.abs(np.sum(vecs[:, :4] * sx[:, :4], axis=0))
        assert np.all(np.abs(dots - 1.0) < 1e-8)


def test_server_cancel_and_budget(H):
    m = G.laplacian_2d(40)
    op = H.dcsrmv_operator_gpu(m)
    srv = H.Server(mem_budget_bytes=8 << 20, max_slots=8)
    a = srv.submit(op, 6, 18)
    b = srv.submit(op, 6, 18)
    srv.cancel(b)
    for _ in range(2000):
        srv.step()
        if srv.poll(a) is not None:
            break
    ra, rb = srv.poll(a), srv.poll(b)
    assert ra is not None and ra[0] == 0
    assert rb is not None and rb[0] == 9       # HLANC_ERR_CANCELLED
    with pytest.raises(H.HLancError):          # larger than the whole budget
        small = H.Server(mem_budget_bytes=1 << 16, max_slots=2)
        small.submit(op, 6, 18)


def test_cpp_dropin_end_to_end(H, tmp_path, readers_golden):
    exe = tmp_path / "demo_dropin"
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                           os.path.join(ROOT, "tests", "cpp", "demo_dropin.cpp"), "-o", str(exe),
                           "-L", os.path.dirname(H.LIB_PATH), "-lhlanc_gb300",
                           f"-Wl,-rpath,{os.path.dirname(H.LIB_PATH)}"])
    # the reference's simple.pp written by our own writer from the golden arrays
    g = readers_golden
    mat = H.dcsr_matrix_t.from_arrays(g["simple_row_ptr"], g["simple_col"], g["simple_val"],
                                      int(g["simple_meta"][1]))
    pp = tmp_path / "simple.pp"
    mat.save_pp(str(pp))
    eigs = tmp_path / "simple.eigs"
    out = subprocess.check_output([str(exe), "pp", str(pp), "4", "12", str(eigs)]).decode().splitlines()
    ref = golden("simple_pp.npz")["values"]
    for line in out:
        parts = line.split()
        kind, rc = parts[0], int(parts[1])
        assert rc == 0, line
        if kind == "eigs":
            assert parts[2:] == ["4", "16"], line
            continue
        vals = np.array([float(x) for x in parts[-4:]])
        assert np.abs(vals - ref).max() <= 1e-10 * np.abs(ref).max(), line
    # the demo's eigs file passes the reference verifier's check (demo/verify_eigs.cu)
    ev, ex = H.read_eigs(str(eigs))
    op = H.dcsrmv_operator_gpu(mat)
    res, rd = H.residuals(op, ev, ex)
    assert rd.max() < 1e-9 and np.abs(ev - ref).max() <= 1e-10 * np.abs(ref).max()


def test_residuals_host_match_device(H, torch):
    m = G.laplacian_2d(30)
    op = H.dcsrmv_operator_gpu(m)
    rc, vals, vecs, st = H.solve(op, 5, 15)
    assert rc == 0
    r_h, d_h = H.residuals(op, vals[:5], vecs[:, :5])
    vd = torch.tensor(vals[:5], dtype=torch.float64, device="cuda")
    xd = torch.tensor(np.ascontiguousarray(vecs[:, :5].T), dtype=torch.float64, device="cuda")
    r_d, d_d = H.residuals_device(op, 5, vd.data_ptr(), xd.data_ptr(), m.n)
    assert np.array_equal(r_h, r_d) and np.array_equal(d_h, d_d)
    assert r_h.max() < 1e-10 * 8


def test_server_mixed_precision_requests(H):
    mats = _batch_mats(6, seed=9, n_lo=1000, n_hi=5000)
    ops = [H.dcsrmv_operator_gpu(m, precision=H.HLANC_PREC_FP32_REFINE) for m in mats]
    srv = H.Server(mem_budget_bytes=64 << 20, max_slots=3)
    ids = [srv.submit(op, 4, 12, precision=H.HLANC_PREC_FP32_REFINE if i % 2 == 0 else H.HLANC_PREC_FP64)
           for i, op in enumerate(ops)]
    results = {}
    for _ in range(5000):
        srv.step()
        for i, rid in enumerate(ids):
            if i not in results:
                r = srv.poll(rid)
                if r is not None:
                    results[i] = r
        if len(results) == len(ids):
            break
    assert len(results) == len(ids)
    for i, m in enumerate(mats):
        status, vals, vecs, st = results[i]
        assert status == 0
        ref = np.sort(np.linalg.eigvalsh(G.to_scipy(m).toarray()))[-4:]
        assert np.abs(vals[:4] - ref).max() <= 1e-10 * np.abs(ref).max()
        R = G.to_scipy(m) @ vecs[:, :4] - vecs[:, :4] * vals[:4]
        assert np.linalg.norm(R, axis=0).max() <= 1e-10 * _norm_a(m)
        if i % 2 == 0:
            assert st["refine_restarts"] >= 1
