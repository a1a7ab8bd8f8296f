"""ctypes binding of the oracle (liboracle.so) and of the reference checker
(_ref/libhlanc_ref.so).  Test infrastructure only; see oracle/__init__.py."""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libhlanc_ref.so")

_lib = None
_ref = None

_i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_f64pF = np.ctypeslib.ndpointer(dtype=np.float64, flags="F_CONTIGUOUS")


class _OCSR(C.Structure):
    _fields_ = [("nrows", C.c_int), ("ncols", C.c_int), ("nnz", C.c_int), ("symmetric", C.c_int),
                ("row_ptr", C.POINTER(C.c_int)), ("col", C.POINTER(C.c_int)),
                ("val", C.POINTER(C.c_double))]


class _Stats(C.Structure):
    _fields_ = [("spmv_calls", C.c_long), ("restarts", C.c_int), ("nconv", C.c_int),
                ("cgs_passes", C.c_long), ("rnorm", C.c_double), ("cycle_seconds", C.c_double),
                ("cycle_spmv", C.c_long), ("cycle_k", C.c_int)]


def build(force: bool = False) -> str:
    """Compile hlanc_oracle.c into liboracle.so (gcc, OpenMP)."""
    src = os.path.join(HERE, "hlanc_oracle.c")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        subprocess.check_call(["gcc", "-O2", "-fopenmp", "-fPIC", "-shared", "-std=c11", src,
                               "-o", LIB_PATH, "-lm"])
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        L.ocsr_from_arrays.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, _i32p, _i32p, _f64p,
                                       C.POINTER(_OCSR)]
        L.ocsr_read.argtypes = [C.c_char_p, C.c_char_p, C.c_int, C.POINTER(_OCSR)]
        for f in ("ocsr_save_pp", "ocsr_save_mm", "ocsr_save_bin"):
            getattr(L, f).argtypes = [C.POINTER(_OCSR), C.c_char_p]
        L.ocsr_free.argtypes = [C.POINTER(_OCSR)]
        L.ocsr_spmv_naive.argtypes = [C.POINTER(_OCSR), _f64p, _f64p]
        L.ocsr_spmv_mkl.argtypes = [C.POINTER(_OCSR), _f64p, _f64p]
        L.ocsr_spmv_general_omp.argtypes = [C.POINTER(_OCSR), _f64p, _f64p]
        L.ocsr_expand_general.argtypes = [C.POINTER(_OCSR), C.POINTER(_OCSR)]
        L.oracle_solve_csr.argtypes = [C.POINTER(_OCSR), C.c_int, C.c_int, _f64p, _f64pF, C.c_int,
                                       _f64p, C.c_double, C.c_int, C.c_int, C.POINTER(_Stats)]
        L.oracle_tridiag_eig.argtypes = [C.c_int, _f64p, _f64p, _f64pF, C.c_int, C.c_int]
        L.oracle_set_threads.argtypes = [C.c_int]
        L.oracle_set_trace.argtypes = [C.c_void_p, C.c_int]
        _lib = L
    return _lib


def _to_ocsr(row_ptr, col, val, ncols, symmetric):
    row_ptr = np.ascontiguousarray(row_ptr, dtype=np.int32)
    col = np.ascontiguousarray(col, dtype=np.int32)
    val = np.ascontiguousarray(val, dtype=np.float64)
    m = _OCSR()
    rc = lib().ocsr_from_arrays(len(row_ptr) - 1, int(ncols), len(col), int(bool(symmetric)),
                                row_ptr, col if len(col) else np.zeros(1, np.int32),
                                val if len(val) else np.zeros(1), C.byref(m))
    if rc:
        raise MemoryError("ocsr_from_arrays failed")
    return m


def _from_ocsr(m: _OCSR):
    n, z = m.nrows, m.nnz
    rp = np.ctypeslib.as_array(m.row_ptr, shape=(n + 1,)).copy()
    ci = np.ctypeslib.as_array(m.col, shape=(max(z, 1),))[:z].copy()
    v = np.ctypeslib.as_array(m.val, shape=(max(z, 1),))[:z].copy()
    return dict(nrows=n, ncols=m.ncols, nnz=z, symmetric=bool(m.symmetric), row_ptr=rp, col=ci, val=v)


def read_matrix(fmt: str, filename: str, symmetric: bool = False) -> dict:
    m = _OCSR()
    rc = lib().ocsr_read(fmt.encode(), filename.encode(), int(symmetric), C.byref(m))
    if rc:
        raise ValueError(f"oracle reader failed ({rc}) on {filename}")
    out = _from_ocsr(m)
    lib().ocsr_free(C.byref(m))
    return out


def save_matrix(fmt: str, filename: str, row_ptr, col, val, ncols, symmetric) -> None:
    m = _to_ocsr(row_ptr, col, val, ncols, symmetric)
    rc = getattr(lib(), f"ocsr_save_{fmt}")(C.byref(m), filename.encode())
    lib().ocsr_free(C.byref(m))
    if rc:
        raise OSError(f"oracle save_{fmt} failed ({rc})")


def spmv(row_ptr, col, val, ncols, symmetric, x, kind: str = "mkl") -> np.ndarray:
    m = _to_ocsr(row_ptr, col, val, ncols, symmetric)
    y = np.zeros(len(row_ptr) - 1)
    fn = {"mkl": lib().ocsr_spmv_mkl, "naive": lib().ocsr_spmv_naive,
          "omp": lib().ocsr_spmv_general_omp}[kind]
    fn(C.byref(m), np.ascontiguousarray(x, dtype=np.float64), y)
    lib().ocsr_free(C.byref(m))
    return y


def solve_csr(row_ptr, col, val, ncols, symmetric, nev, ncv, start, tol=0.0, max_iter=0,
              threads=1, ldv=None, trace=False):
    """Run the oracle ds_solver.  Returns (rc, values[ncv], vectors (ldv x ncv), stats).
    stats['cycle_*'] describe the last restart cycle; with trace=True,
    stats['trace'] lists (seconds, operator applications, first step) per cycle."""
    n = len(row_ptr) - 1
    ldv = n if ldv is None else ldv
    m = _to_ocsr(row_ptr, col, val, ncols, symmetric)
    values = np.zeros(ncv)
    vectors = np.zeros((ldv, ncv), order="F")
    st = _Stats()
    cap = (max_iter if max_iter > 0 else 200) + 1
    buf = np.zeros(3 * cap) if trace else None
    if trace:
        lib().oracle_set_trace(buf.ctypes.data, cap)
    try:
        rc = lib().oracle_solve_csr(C.byref(m), nev, ncv, values, vectors, ldv,
                                    np.ascontiguousarray(start, dtype=np.float64), float(tol),
                                    int(max_iter), int(threads), C.byref(st))
    finally:
        if trace:
            lib().oracle_set_trace(None, 0)
    lib().ocsr_free(C.byref(m))
    stats = dict(spmv_calls=st.spmv_calls, restarts=st.restarts, nconv=st.nconv,
                 cgs_passes=st.cgs_passes, rnorm=st.rnorm, cycle_seconds=st.cycle_seconds,
                 cycle_spmv=st.cycle_spmv, cycle_k=st.cycle_k)
    if trace:
        stats["trace"] = buf.reshape(cap, 3)[:st.restarts].tolist()
    return rc, values, vectors, stats


def tridiag_eig(d, e, want_z=True):
    d = np.array(d, dtype=np.float64)
    e = np.array(e, dtype=np.float64)
    n = d.size
    z = np.zeros((n, n), order="F")
    rc = lib().oracle_tridiag_eig(n, d, e if e.size else np.zeros(1), z, n, int(want_z))
    return rc, d, z


# ---------------------------------------------------------------- reference --
def ref_available() -> bool:
    return os.path.exists(REF_PATH)


def ref_lib():
    global _ref
    if _ref is None:
        R = C.CDLL(REF_PATH)
        R.ref_solve_csr.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, _i32p, _i32p, _f64p,
                                    C.c_int, C.c_int, _f64p, _f64p, _f64pF, C.c_int,
                                    C.POINTER(C.c_long)]
        R.ref_spmv_csr.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, _i32p, _i32p, _f64p,
                                   _f64p, _f64p, C.c_int]
        R.ref_read.argtypes = [C.c_char_p, C.c_char_p, C.c_int] + [C.POINTER(C.c_int)] * 4
        R.ref_read_copy.argtypes = [_i32p, _i32p, _f64p]
        R.ref_save.argtypes = [C.c_char_p, C.c_char_p]
        _ref = R
    return _ref


def ref_solve_csr(row_ptr, col, val, ncols, symmetric, nev, ncv, start, ldv=None):
    n = len(row_ptr) - 1
    ldv = n if ldv is None else ldv
    values = np.zeros(ncv)
    vectors = np.zeros((ldv, ncv), order="F")
    calls = C.c_long(0)
    z = len(col)
    rc = ref_lib().ref_solve_csr(n, int(ncols), z, int(bool(symmetric)),
                                 np.ascontiguousarray(row_ptr, dtype=np.int32),
                                 np.ascontiguousarray(col, dtype=np.int32) if z else np.zeros(1, np.int32),
                                 np.ascontiguousarray(val, dtype=np.float64) if z else np.zeros(1),
                                 nev, ncv, np.ascontiguousarray(start, dtype=np.float64),
                                 values, vectors, ldv, C.byref(calls))
    return rc, values, vectors, calls.value


def ref_spmv(row_ptr, col, val, ncols, symmetric, x, naive=False):
    n = len(row_ptr) - 1
    y = np.zeros(n)
    z = len(col)
    ref_lib().ref_spmv_csr(n, int(ncols), z, int(bool(symmetric)),
                           np.ascontiguousarray(row_ptr, dtype=np.int32),
                           np.ascontiguousarray(col, dtype=np.int32) if z else np.zeros(1, np.int32),
                           np.ascontiguousarray(val, dtype=np.float64) if z else np.zeros(1),
                           np.ascontiguousarray(x, dtype=np.float64), y, int(naive))
    return y


def ref_read(fmt: str, filename: str, symmetric: bool = False) -> dict:
    R = ref_lib()
    n, c, z, s = C.c_int(), C.c_int(), C.c_int(), C.c_int()
    R.ref_read(fmt.encode(), filename.encode(), int(symmetric), C.byref(n), C.byref(c),
               C.byref(z), C.byref(s))
    rp = np.zeros(n.value + 1, np.int32)
    ci = np.zeros(max(z.value, 1), np.int32)
    v = np.zeros(max(z.value, 1))
    R.ref_read_copy(rp, ci, v)
    return dict(nrows=n.value, ncols=c.value, nnz=z.value, symmetric=bool(s.value), row_ptr=rp,
                col=ci[:z.value], val=v[:z.value])


def ref_save(fmt: str, filename: str) -> None:
    if ref_lib().ref_save(fmt.encode(), filename.encode()):
        raise OSError("ref_save failed")
