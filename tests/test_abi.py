"""C-ABI checks that need no GPU: every symbol include/hlanc_gb300.h
declares is exported, the Python struct layouts match the C ones, the
host-side readers/writers are bit-exact with the reference's, and the C++
drop-in header compiles with the reference demo's calls."""
import ctypes as C
import os
import re
import shutil
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, ROOT

INC = os.path.join(ROOT, "include")


@pytest.fixture(scope="module")
def H():
    import hlanc_gb300 as H
    from hlanc_gb300 import build
    build.build()
    return H


def _declared():
    text = open(os.path.join(INC, "hlanc_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(hlanc_[a-z0-9_]+)\s*\(", text)))


def test_exports_every_declared_symbol(H):
    names = _declared()
    assert len(names) >= 25
    L = C.CDLL(H.LIB_PATH)
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_struct_layouts_match(H, tmp_path):
    src = tmp_path / "sz.c"
    src.write_text('#include "hlanc_gb300.h"\n#include <stdio.h>\n#include <stddef.h>\n'
                   'int main(void){printf("%zu %zu %zu %zu %zu\\n", sizeof(hlanc_opts_t), sizeof(hlanc_stats_t),'
                   ' sizeof(hlanc_profile_t), sizeof(hlanc_server_opts_t), offsetof(hlanc_opts_t, profile));return 0;}\n')
    exe = tmp_path / "sz"
    subprocess.check_call(["gcc", "-I", INC, str(src), "-o", str(exe)])
    out = subprocess.check_output([str(exe)]).decode().split()
    assert [int(x) for x in out] == [C.sizeof(H.Opts), C.sizeof(H.Stats), C.sizeof(H.Profile),
                                     C.sizeof(H.ServerOpts), H.Opts.profile.offset]


def test_cgs_diag_rejects_bad_arguments(H):
    # argument checks come before any CUDA call
    ms = (C.c_double * 3)()
    f = H.lib().hlanc_diag_cgs
    bad = 2                                                         # HLANC_ERR_INVALID
    assert f(0, 100, 8, H.HLANC_CGS_HYBRID, 1, ms) == bad         # n < 1024
    assert f(0, 4096, 1, H.HLANC_CGS_HYBRID, 1, ms) == bad        # c < 2
    assert f(0, 4096, 8, H.HLANC_CGS_AUTO, 1, ms) == bad          # mode must be FP64 or HYBRID
    assert f(0, 4096, H.HLANC_MAX_NCV + 1, H.HLANC_CGS_FP64, 1, ms) == bad
    assert f(0, 4096, 8, H.HLANC_CGS_FP64, 1, None) == bad


def test_operator_rejects_bad_csr_before_any_cuda_call(H):
    # 2^17 rows: the checks run in row chunks on the host worker pool; a bad
    # row pointer or column index in any chunk is found before device memory
    # is touched (HLANC_ERR_INVALID), and a valid matrix gets past them
    n = 1 << 17
    rp = (np.arange(n + 1) * 2).astype(np.int32)
    col = np.stack([np.arange(n), (np.arange(n) + 1) % n], axis=1).reshape(-1).astype(np.int32)
    val = np.ones(2 * n)
    f = H.lib().hlanc_csr_create

    def create(rp_, col_, nnz):
        h = C.c_void_p()
        rc = f(0, n, n, nnz, rp_.ctypes.data, col_.ctypes.data, val.ctypes.data, 0, H.HLANC_PREC_FP64, C.byref(h))
        if rc == 0:
            H.lib().hlanc_csr_destroy(h)
        return rc

    bad = 2                                                         # HLANC_ERR_INVALID
    r = rp.copy()
    r[n - 5] = r[n - 6] - 1                                         # decreasing, in the last chunk
    assert create(r, col, 2 * n) == bad
    c = col.copy()
    c[-3] = n                                                       # column out of range, last chunk
    assert create(rp, c, 2 * n) == bad
    c = col.copy()
    c[7] = -1                                                       # negative column, first chunk
    assert create(rp, c, 2 * n) == bad
    assert create(rp, col, 2 * n - 1) == bad                        # row_ptr[n] > nnz
    assert create(rp, col, 2 * n) in (0, 3)                         # ok, or no device here (HLANC_ERR_CUDA)


def test_status_strings(H):
    assert H.lib().hlanc_status_string(0) == b"ok"
    assert H.lib().hlanc_status_string(1) == b"not converged"


def test_readers_bit_exact_through_abi(H, readers_golden, tmp_path):
    g = readers_golden
    i = 0
    while f"c{i}_meta" in g:
        fmt, fn, sym = str(g[f"c{i}_case"]).split("|")
        m = H.dcsr_matrix_t(fmt, os.path.join(GOLDEN, "readers", fn), bool(int(sym)))
        assert [m.get_num_rows(), m.get_num_columns(), m.get_nnz(), int(m.symmetric())] == list(g[f"c{i}_meta"])
        assert np.array_equal(m.get_row_ptr(), g[f"c{i}_row_ptr"])
        assert np.array_equal(m.get_column_index(), g[f"c{i}_col"])
        assert np.array_equal(m.get_value(), g[f"c{i}_val"])
        for wfmt in ("pp", "mm", "bin"):
            key = f"c{i}_save_{wfmt}"
            if key not in g:
                continue
            out = tmp_path / f"c{i}.{wfmt}"
            getattr(m, f"save_{wfmt}")(str(out))
            assert np.array_equal(np.frombuffer(out.read_bytes(), np.uint8), g[key]), (fn, wfmt)
        i += 1
    assert i >= 8


def test_bin_roundtrip_of_symmetric(H, readers_golden, tmp_path):
    g = readers_golden
    m = H.dcsr_matrix_t.from_arrays(g["journals_row_ptr"], g["journals_col"], g["journals_val"],
                                    int(g["journals_meta"][1]), True)
    p = tmp_path / "j.bin"
    m.save_bin(str(p))
    b = H.dcsr_matrix_t("bin", str(p))
    assert not b.symmetric()
    assert np.array_equal(b.get_row_ptr(), g["journals_bin_row_ptr"])
    assert np.array_equal(b.get_column_index(), g["journals_bin_col"])
    assert np.array_equal(b.get_value(), g["journals_bin_val"])


def test_reader_errors_are_status_codes(H, tmp_path):
    bad = tmp_path / "bad.mtx"
    bad.write_text("%%MatrixMarket matrix array real general\n2 2\n1\n2\n3\n4\n")
    with pytest.raises(H.HLancError) as e:
        H.dcsr_matrix_t("mm", str(bad))
    assert e.value.status == 6
    with pytest.raises(H.HLancError):
        H.dcsr_matrix_t("mm", str(tmp_path / "missing.mtx"))
    crlf = tmp_path / "crlf.pp"
    crlf.write_bytes(b"0:1 1:2\r\n")
    with pytest.raises(H.HLancError):
        H.dcsr_matrix_t("pp", str(crlf))
    with pytest.raises(H.HLancError):
        H.dcsr_matrix_t("xyz", str(crlf))


@pytest.mark.skipif(shutil.which("g++") is None, reason="g++ missing")
def test_cpp_header_compiles_with_reference_demo_calls(tmp_path):
    exe = tmp_path / "demo"
    subprocess.check_call(["g++", "-std=c++17", "-fsyntax-only", "-Wall", "-Wextra", "-I", INC,
                           os.path.join(ROOT, "tests", "cpp", "demo_dropin.cpp")])
