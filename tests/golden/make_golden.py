"""Write the golden fixtures under tests/golden/ from the reference's own CPU
path (ds_solver_mkl + dcsrmv_operator_mkl + dcsr_matrix_t, compiled by
oracle/build_ref.sh into oracle/_ref/libhlanc_ref.so).

Run in a container where the reference sources are mounted:

    ./oracle/build_ref.sh && python tests/golden/make_golden.py REFERENCE_DIR
    python tests/golden/make_golden.py --large   # 2^18-row cases (about a minute)
    python tests/golden/make_golden.py --full    # full-size C2/C3 eigenvalues (tens of minutes)

Every solve starts from the generators' seeded start vector (the MKL shim
injects it where the reference calls dlarnv), so the fixtures, the oracle and
the GPU library all begin from the same vector.  Reader fixtures are small
text files written by this script (readers/*.pp, readers/*.mtx) plus the
reference's CSR arrays for them and its writer outputs.
"""
from __future__ import annotations

import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle as O  # noqa: E402
from hlanc_gb300 import generators as G  # noqa: E402

READERS = os.path.join(HERE, "readers")


def fingerprint(rp, ci, v):
    """Structure and value checksums of a CSR matrix: a test regenerates the
    matrix from its generator and compares these before it compares
    eigenvalues, so a generator change cannot pass as a solver change."""
    rp, ci, v = np.asarray(rp, np.int64), np.asarray(ci, np.int64), np.asarray(v, np.float64)
    w = np.arange(1, ci.size + 1, dtype=np.float64)
    return np.array([rp.size - 1, ci.size, float(ci.sum()), float((ci * (np.arange(ci.size) % 7)).sum()),
                     float(v.sum()), float(np.abs(v).sum()), float((v * w).sum() / ci.size)])


def solve_case(name, m, nev, ncv, symmetric=False, seed=0, keep_vectors=False, **extra):
    x0 = G.start_vector(m.n if hasattr(m, "n") else len(m["row_ptr"]) - 1, seed)
    if isinstance(m, dict):
        rp, ci, v, nc = m["row_ptr"], m["col"], m["val"], m["ncols"]
    else:
        rp, ci, v, nc = m.row_ptr, m.col, m.val, m.ncols
    t0 = time.perf_counter()
    rc, vals, vecs, calls = O.ref_solve_csr(rp, ci, v, nc, symmetric, nev, ncv, x0)
    dt = time.perf_counter() - t0
    assert rc == 0, (name, rc)
    out = dict(values=vals[:nev], nev=nev, ncv=ncv, seed=seed, spmv_calls=calls, symmetric=symmetric,
               fingerprint=fingerprint(rp, ci, v), ref_seconds=dt, ref_threads=os.cpu_count() or 1)
    if keep_vectors:
        out["vectors"] = np.ascontiguousarray(vecs[:, :nev])
    out.update(extra)
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
    print(f"{name}: rc={rc} spmv={calls} top={vals[nev - 1]:.15g} ({dt:.1f} s)", flush=True)


def write_reader_inputs():
    os.makedirs(READERS, exist_ok=True)
    files = {
        # blank-separated tokens, a zero value, an empty row, tabs, a final
        # row without newline (its entries land in col/val without a row_ptr)
        "plain.pp": "0:4 1:-1\n0:-1 1:4\t2:-1 3:0\n\n1:-1 2:4\n2:2.5 3:1e-3 5:7",
        # symmetric reading drops upper entries and widens num_columns
        "upper.pp": "0:2 1:1 2:3\n0:1 1:2\n0:3 1:0 2:5\n",
        "trailing_blank.pp": "0:1  \n 1:2\n\n",
        "general.mtx": ("%%MatrixMarket matrix coordinate real general\n% comment line\n%another\n"
                        "4 5 7\n1 1 1.5\n3 2 -2\n1 4 3\n2 2 0\n4 5 9.25\n3 1 4\n1 2 -1\n"),
        "symmetric.mtx": ("%%MatrixMarket matrix coordinate real symmetric\n4 4 6\n"
                          "1 1 2\n2 1 -1\n2 2 2\n3 2 -1\n1 3 7\n4 4 0\n"),
        "integer_sym.mtx": ("%%MatrixMarket matrix coordinate integer symmetric\n3 3 4\n"
                            "1 1 3\n2 1 1\n3 3 5\n3 1 2\n"),
    }
    for fn, text in files.items():
        with open(os.path.join(READERS, fn), "w") as f:
            f.write(text)
    return files


def reader_fixtures(ref_dir):
    write_reader_inputs()
    cases = [("pp", "plain.pp", False), ("pp", "plain.pp", True), ("pp", "upper.pp", True),
             ("pp", "upper.pp", False), ("pp", "trailing_blank.pp", False),
             ("mm", "general.mtx", False), ("mm", "symmetric.mtx", False),
             ("mm", "integer_sym.mtx", False)]
    out = {}
    tmp = os.path.join("/tmp", f"hlanc_golden_{os.getpid()}")
    os.makedirs(tmp, exist_ok=True)
    for i, (fmt, fn, sym) in enumerate(cases):
        d = O.ref_read(fmt, os.path.join(READERS, fn), sym)
        key = f"c{i}"
        out[f"{key}_meta"] = np.array([d["nrows"], d["ncols"], d["nnz"], int(d["symmetric"])])
        out[f"{key}_row_ptr"] = d["row_ptr"]
        out[f"{key}_col"] = d["col"]
        out[f"{key}_val"] = d["val"]
        out[f"{key}_case"] = np.array(f"{fmt}|{fn}|{int(sym)}")
        for wfmt in ("pp", "mm", "bin"):
            path = os.path.join(tmp, f"{key}.{wfmt}")
            if d["nrows"] == 0:
                continue
            O.ref_save(wfmt, path)
            with open(path, "rb") as f:
                out[f"{key}_save_{wfmt}"] = np.frombuffer(f.read(), dtype=np.uint8)
    # the reference's data files
    for tag, fmt, fn in (("simple", "pp", "data/simple.pp"), ("journals", "mm", "data/Journals.mtx")):
        path = os.path.join(ref_dir, fn)
        d = O.ref_read(fmt, path, False)
        out[f"{tag}_meta"] = np.array([d["nrows"], d["ncols"], d["nnz"], int(d["symmetric"])])
        out[f"{tag}_row_ptr"], out[f"{tag}_col"], out[f"{tag}_val"] = d["row_ptr"], d["col"], d["val"]
        binp = os.path.join(tmp, f"{tag}.bin")
        O.ref_save("bin", binp)
        b = O.ref_read("bin", binp, False)
        out[f"{tag}_bin_row_ptr"], out[f"{tag}_bin_col"], out[f"{tag}_bin_val"] = b["row_ptr"], b["col"], b["val"]
        out[f"{tag}_bin_meta"] = np.array([b["nrows"], b["ncols"], b["nnz"], int(b["symmetric"])])
    np.savez_compressed(os.path.join(HERE, "readers.npz"), **out)
    print("readers.npz:", len(cases), "reader cases")
    return out


def spmv_fixture(readers):
    rp, ci, v = readers["journals_row_ptr"], readers["journals_col"], readers["journals_val"]
    n = len(rp) - 1
    x = G.uniform_pm1(7, 0, n)
    y_mkl = O.ref_spmv(rp, ci, v, n, True, x, naive=False)
    y_naive = O.ref_spmv(rp, ci, v, n, True, x, naive=True)
    lap = G.laplacian_2d(7, 5)
    x2 = G.uniform_pm1(8, 0, lap.n)
    y2 = O.ref_spmv(lap.row_ptr, lap.col, lap.val, lap.ncols, False, x2, naive=False)
    np.savez_compressed(os.path.join(HERE, "spmv.npz"), x_sym=x, y_sym_mkl=y_mkl, y_sym_naive=y_naive,
                        x_gen=x2, y_gen=y2)
    print("spmv.npz")


def large_cases():
    """Sizes where the library's default kernels differ from the small cases:
    launches over >= 2^18 rows take the hybrid (FP64 + fixed-point) CGS
    kernels and the tensor-core basis update.  About a minute on 8 cores."""
    solve_case("lap3d_64_shift", G.laplacian_3d(64, shift_seed=1), 20, 60)
    solve_case("chunglu_2e18", G.chung_lu_normalized(1 << 18, seed=2), 16, 48)


def full_cases():
    """Eigenvalues of the two single-solve workloads at full size (3-D
    Laplacian 160^3 + shift, nev 20, ncv 60; Chung-Lu n = 2^22, nev 16,
    ncv 48).  Tens of minutes on 8 cores; values only."""
    solve_case("c3_chunglu_2e22", G.chung_lu_normalized(1 << 22, seed=2), 16, 48)
    solve_case("c2_lap3d_160_shift", G.laplacian_3d(160, shift_seed=1), 20, 60)


def main():
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    flags = {a for a in sys.argv[1:] if a.startswith("--")}
    ref_dir = args[0] if args else os.environ.get("HLANC_REFERENCE")
    if not O.ref_available():
        sys.exit("oracle/_ref/libhlanc_ref.so missing: run oracle/build_ref.sh first")
    if "--large" in flags:
        large_cases()
        return
    if "--full" in flags:
        full_cases()
        return
    if not ref_dir:
        sys.exit("usage: make_golden.py REFERENCE_DIR | --large | --full (or set HLANC_REFERENCE)")
    readers = reader_fixtures(ref_dir)
    spmv_fixture(readers)
    # the demo's cases (demo/HLanc_demo.cu): nev=4, ncv=12
    simple = dict(row_ptr=readers["simple_row_ptr"], col=readers["simple_col"], val=readers["simple_val"],
                  ncols=int(readers["simple_meta"][1]))
    solve_case("simple_pp", simple, 4, 12, symmetric=False, keep_vectors=True)
    journals = dict(row_ptr=readers["journals_row_ptr"], col=readers["journals_col"],
                    val=readers["journals_val"], ncols=int(readers["journals_meta"][1]))
    solve_case("journals_mtx", journals, 4, 12, symmetric=True, keep_vectors=True)
    # workload generators at CPU-feasible sizes
    solve_case("c1_laplacian2d_100", G.laplacian_2d(100), 10, 30)
    solve_case("lap3d_12_shift", G.laplacian_3d(12, shift_seed=1), 20, 60)
    solve_case("banded_3000_bw5", G.banded_random(3000, 5, seed=3, problem=0), 8, 24)
    solve_case("chunglu_4096", G.chung_lu_normalized(4096, seed=2), 16, 48)
    solve_case("lap2d_odd_37x23", G.laplacian_2d(37, 23), 6, 20, seed=5, keep_vectors=True)


if __name__ == "__main__":
    main()
