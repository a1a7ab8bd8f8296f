"""A whole Lanczos extension in one cooperative launch (HLANC_CYCLE_AUTO on
small problems, kernels_cycle.cu) against the reference's CPU solver
(golden fixtures) and against the per-phase launches of the same solve.
The two paths sum their reductions in different orders, so they agree to
rounding, not bit for bit: eigenvalues within 1e-10 relative of the
reference, and of each other."""
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


def _used(H, before):
    return {k: v - before[k] for k, v in H.variant_counts().items()}


@pytest.mark.parametrize("case,gen,nev,ncv,mixed", [
    ("c1_laplacian2d_100", lambda: G.laplacian_2d(100), 10, 30, False),
    ("lap3d_12_shift", lambda: G.laplacian_3d(12, shift_seed=1), 20, 60, False),
    ("banded_3000_bw5", lambda: G.banded_random(3000, 5, seed=3, problem=0), 8, 24, False),
    ("banded_3000_bw5", lambda: G.banded_random(3000, 5, seed=3, problem=0), 8, 24, True),
])
def test_one_launch_extension_matches_reference(H, case, gen, nev, ncv, mixed):
    """Eligible problems (rows of <= 96 entries, few rows) take the one-launch
    extension by default, in FP64 and in mixed precision."""
    g = golden(f"{case}.npz")
    m = gen()
    prec = H.HLANC_PREC_FP32_REFINE if mixed else H.HLANC_PREC_FP64
    op = H.dcsrmv_operator_gpu(m, precision=prec)
    before = H.variant_counts()
    rc, vals, vecs, st = H.solve(op, nev, ncv, seed=int(g["seed"]), precision=prec)
    used = _used(H, before)
    assert rc == 0, st
    ref = g["values"]
    assert np.abs(vals[:nev] - ref).max() <= EV_RTOL * np.abs(ref).max()
    A = G.to_scipy(m)
    R = A @ vecs[:, :nev] - vecs[:, :nev] * vals[:nev]
    assert np.linalg.norm(R, axis=0).max() <= 1e-10 * np.abs(A).sum(axis=1).max()
    assert used["cycle"] > 0 and used["proj_fp64"] == 0 and used["proj_hybrid"] == 0, used
    # the per-phase launches of the same solve
    rc2, vals2, _, st2 = H.solve(op, nev, ncv, seed=int(g["seed"]), precision=prec, cycle=H.HLANC_CYCLE_OFF)
    assert rc2 == 0
    assert np.abs(vals2[:nev] - vals[:nev]).max() <= EV_RTOL * np.abs(ref).max()


def test_one_launch_extension_for_a_batch_and_a_server(H):
    import torch
    mats = [G.laplacian_2d(40, 30), G.banded_random(3000, 4, seed=3, problem=1), G.laplacian_3d(14, shift_seed=2)]
    ops = [H.dcsrmv_operator_gpu(m) for m in mats]
    solo = [H.solve(op, 6, 18)[1][:6] for op in ops]
    outs = [(torch.zeros(18, dtype=torch.float64, device="cuda"),
             torch.zeros((18, m.n), dtype=torch.float64, device="cuda")) for m in mats]
    before = H.variant_counts()
    b = H.Batch(ops, 6, 18)
    status, st = b.run([v.data_ptr() for v, _ in outs], [x.data_ptr() for _, x in outs])
    b.close()
    assert (status == 0).all()
    assert _used(H, before)["cycle"] > 0
    for (v, _), ref in zip(outs, solo):
        assert np.abs(v[:6].cpu().numpy() - ref).max() <= 1e-10 * np.abs(ref).max()
    srv = H.Server(mem_budget_bytes=1 << 30, max_slots=8)
    ids = [srv.submit(op, 6, 18) for op in ops]
    res = {}
    while len(res) < len(ids):
        srv.step()
        for rid in ids:
            if rid not in res:
                r = srv.poll(rid)
                if r is not None:
                    res[rid] = r
    srv.close()
    for rid, ref in zip(ids, solo):
        assert res[rid][0] == 0
        assert np.abs(res[rid][1][:6] - ref).max() <= 1e-10 * np.abs(ref).max()


def test_long_rows_keep_per_phase_launches(H):
    g = golden("chunglu_4096.npz")
    m = G.chung_lu_normalized(4096, seed=2)
    op = H.dcsrmv_operator_gpu(m)
    before = H.variant_counts()
    rc, vals, _, _ = H.solve(op, 16, 48, seed=int(g["seed"]))
    assert rc == 0 and _used(H, before)["cycle"] == 0
    assert np.abs(vals[:16] - g["values"]).max() <= EV_RTOL * np.abs(g["values"]).max()


def test_group_barrier_timeout_reaches_caller(H):
    # more than one CTA in the group, and barrier waits that give up at once
    m = G.laplacian_2d(60, 40)
    op = H.dcsrmv_operator_gpu(m)
    with pytest.raises(H.HLancError) as e:
        H.solve(op, 6, 18, wait_limit=-1)
    assert e.value.status == 5
    rc, vals, _, _ = H.solve(op, 6, 18)
    assert rc == 0
    ana = G.laplacian_2d_eigenvalues(60, 40)[-6:]
    assert np.abs(vals[:6] - ana).max() < 1e-10 * 8
