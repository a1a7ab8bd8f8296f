"""hlanc_gb300 -- GB300 (sm_103a) implicitly restarted Lanczos, Python host mirror.

Mirrors the reference's C++ interface (butterfly0923/HLanc, HLanc.hpp):

    m  = dcsr_matrix_t("mm", "Journals.mtx")          # HLanc.hpp:74-392
    op = dcsrmv_operator_gpu(m, dev=0)                 # HLanc.hpp:476-572
    rc = ds_solver_gpu(n, nev, ncv, values, vectors, ldv, op, dev=0)   # HLanc.hpp:1868

with the same argument meaning and return values (0 = success, 1 = fewer
than nev converged).  Errors of the library itself raise HLancError.  Every
call goes through the C ABI of libhlanc_gb300.so (include/hlanc_gb300.h);
there is no CPU fallback: if the library is missing, loading fails loudly.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Callable, Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libhlanc_gb300.so")

HLANC_OK = 0
HLANC_NOT_CONVERGED = 1
HLANC_PREC_FP64 = 0
HLANC_PREC_FP32_REFINE = 1
HLANC_BASIS_AUTO = 0
HLANC_BASIS_FP64 = 1
HLANC_CGS_AUTO = 0
HLANC_CGS_FP64 = 1
HLANC_CGS_HYBRID = 2
CGS_HYBRID_MIN_ROWS = 1 << 18     # HLANC_CGS_AUTO picks the hybrid kernels from this many rows
HLANC_MAX_NCV = 128
HLANC_MAX_NEV = 63
# kernel variants counted by hlanc_kernel_launches_of
(KL_ALL, KL_PROJ_HYBRID, KL_PROJ_FP64, KL_APPLY_SHADOW, KL_APPLY_FP64, KL_BASIS_TC, KL_BASIS_FP64, KL_CYCLE,
 KL_RITZ_TC, KL_RITZ_FP64) = range(10)
HLANC_CYCLE_AUTO = 0
HLANC_CYCLE_OFF = 1

_lib = None


class HLancError(RuntimeError):
    def __init__(self, status: int, what: str = ""):
        msg = lib().hlanc_status_string(status).decode() if _lib is not None else str(status)
        super().__init__(f"{what}: status {status} ({msg})" if what else f"status {status} ({msg})")
        self.status = status


class Opts(C.Structure):
    _fields_ = [("tol", C.c_double), ("max_restarts", C.c_int), ("precision", C.c_int),
                ("seed", C.c_ulonglong), ("start", C.POINTER(C.c_double)), ("stream", C.c_void_p),
                ("use_graphs", C.c_int), ("restart_on_device", C.c_int), ("profile", C.c_int),
                ("basis_kernel", C.c_int), ("cgs_kernel", C.c_int), ("wait_limit", C.c_int),
                ("cycle_kernel", C.c_int), ("reserved", C.c_int * 1)]


class Stats(C.Structure):
    _fields_ = [("spmv_calls", C.c_longlong), ("cgs_passes", C.c_longlong), ("restarts", C.c_int),
                ("nconv", C.c_int), ("refine_restarts", C.c_int), ("status", C.c_int),
                ("rnorm", C.c_double), ("seconds", C.c_double), ("bytes_spmv", C.c_double),
                ("bytes_cgs", C.c_double), ("bytes_restart", C.c_double), ("cgs_update_fp32_share", C.c_double),
                ("refine_residual", C.c_double), ("copy_out_seconds", C.c_double), ("reserved", C.c_double * 1)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "reserved"}


PROF_CLASSES = ("spmv", "cgs_proj", "cgs_apply", "basis", "ritz", "aux", "host_restart", "cycle")


class Profile(C.Structure):
    _fields_ = [("launches", C.c_longlong * 8), ("ms", C.c_double * 8), ("bytes", C.c_double * 8),
                ("flops", C.c_double * 8)]

    def as_dict(self) -> dict:
        return {name: dict(launches=self.launches[i], ms=self.ms[i], bytes=self.bytes[i], flops=self.flops[i])
                for i, name in enumerate(PROF_CLASSES)}


class ServerOpts(C.Structure):
    _fields_ = [("mem_budget_bytes", C.c_size_t), ("max_slots", C.c_int), ("dev", C.c_int), ("lanes", C.c_int)]


class ServerStats(C.Structure):
    _fields_ = [("steps", C.c_longlong), ("cycles", C.c_longlong), ("admitted", C.c_longlong),
                ("retired", C.c_longlong), ("wall_ms", C.c_double), ("wait_ms", C.c_double),
                ("host_ms", C.c_double), ("launch_ms", C.c_double), ("admin_ms", C.c_double),
                ("gpu_ms", C.c_double), ("reserved", C.c_double * 6)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "reserved"}


HOST_OP = C.CFUNCTYPE(C.c_int, C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double))

_p = C.c_void_p
_i = C.c_int
_ip = C.POINTER(C.c_int)
_dp = C.POINTER(C.c_double)


def _declare(L):
    sig = {
        "hlanc_status_string": (C.c_char_p, [_i]),
        "hlanc_version": (_i, [_ip, _ip]),
        "hlanc_kernel_launches": (C.c_longlong, []),
        "hlanc_kernel_launches_of": (C.c_longlong, [_i]),
        "hlanc_opts_default": (None, [C.POINTER(Opts)]),
        "hlanc_matrix_read": (_i, [C.c_char_p, C.c_char_p, _i, C.POINTER(_p)]),
        "hlanc_matrix_create": (_i, [_i, _i, _i, _p, _p, _p, _i, C.POINTER(_p)]),
        "hlanc_matrix_info": (_i, [_p, _ip, _ip, _ip, _ip]),
        "hlanc_matrix_arrays": (_i, [_p, C.POINTER(_ip), C.POINTER(_ip), C.POINTER(_dp)]),
        "hlanc_matrix_save": (_i, [_p, C.c_char_p, C.c_char_p]),
        "hlanc_matrix_destroy": (_i, [_p]),
        "hlanc_csr_create": (_i, [_i, _i, _i, _i, _p, _p, _p, _i, _i, C.POINTER(_p)]),
        "hlanc_csr_destroy": (_i, [_p]),
        "hlanc_csr_info": (_i, [_p, _ip, _ip, _ip, C.POINTER(C.c_longlong), _ip]),
        "hlanc_csr_apply": (_i, [_p, _p, _p]),
        "hlanc_csr_spmv_async": (_i, [_p, _p, _p, _p]),
        "hlanc_csr_spmv_f32_async": (_i, [_p, _p, _p, _p]),
        "hlanc_csr_tuning": (_i, [_p, _ip, _ip, _ip, _dp, _dp]),
        "hlanc_solve": (_i, [_i, _i, _i, _i, _p, _p, _i, _p, HOST_OP, _p, C.POINTER(Opts),
                             C.POINTER(Stats)]),
        "hlanc_solve_device": (_i, [_i, _i, _i, _i, _p, _p, _i, _p, C.POINTER(Opts), C.POINTER(Stats)]),
        "hlanc_residuals_device": (_i, [_p, _i, _p, _p, _i, _p, _p]),
        "hlanc_residuals_host": (_i, [_p, _i, _p, _p, _i, _p, _p]),
        "hlanc_eigs_write": (_i, [C.c_char_p, _i, _i, _p, _p, _i]),
        "hlanc_eigs_info": (_i, [C.c_char_p, _ip, _ip]),
        "hlanc_eigs_read": (_i, [C.c_char_p, _p, _p, _i]),
        "hlanc_last_profile": (_i, [C.POINTER(Profile)]),
        "hlanc_diag_fp64_tflops": (_i, [_i, C.POINTER(C.c_double)]),
        "hlanc_diag_cgs": (_i, [_i, _i, _i, _i, _i, C.POINTER(C.c_double)]),
        "hlanc_batch_create": (_i, [_i, _i, _p, _p, _p, C.POINTER(Opts), C.POINTER(_p)]),
        "hlanc_batch_run": (_i, [_p, _p, _p, _p, C.POINTER(Stats)]),
        "hlanc_batch_destroy": (_i, [_p]),
        "hlanc_server_create": (_i, [C.POINTER(ServerOpts), C.POINTER(_p)]),
        "hlanc_server_submit": (_i, [_p, _p, _i, _i, C.POINTER(Opts), C.POINTER(C.c_longlong)]),
        "hlanc_server_step": (_i, [_p, _ip, _ip]),
        "hlanc_server_poll": (_i, [_p, C.c_longlong, _ip, _ip, _p, _p, C.POINTER(Stats)]),
        "hlanc_server_cancel": (_i, [_p, C.c_longlong]),
        "hlanc_server_stats": (_i, [_p, C.POINTER(ServerStats)]),
        "hlanc_server_destroy": (_i, [_p]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    return L


def lib():
    """The loaded C-ABI library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: build it with hlanc_gb300.build.build()")
        _lib = _declare(C.CDLL(LIB_PATH))
    return _lib


def _check(rc: int, what: str) -> None:
    if rc != HLANC_OK:
        raise HLancError(rc, what)


def opts(tol: float = 0.0, max_restarts: int = 200, precision: int = HLANC_PREC_FP64, seed: int = 0,
         start: Optional[np.ndarray] = None, stream: int = 0, use_graphs: bool = True,
         restart_on_device: bool = False, profile: bool = False, basis_fp64: bool = False,
         cgs: int = HLANC_CGS_AUTO, wait_limit: int = 0, cycle: int = 0):
    o = Opts()
    lib().hlanc_opts_default(C.byref(o))
    o.basis_kernel = HLANC_BASIS_FP64 if basis_fp64 else HLANC_BASIS_AUTO
    o.cgs_kernel = cgs
    o.wait_limit = wait_limit
    o.cycle_kernel = cycle
    o.tol, o.max_restarts, o.precision, o.seed = tol, max_restarts, precision, seed
    o.use_graphs = int(use_graphs)
    o.restart_on_device = int(restart_on_device)
    o.profile = int(profile)
    o.stream = stream or None
    keep = None
    if start is not None:
        keep = np.ascontiguousarray(start, dtype=np.float64)
        o.start = keep.ctypes.data_as(_dp)
    return o, keep


# ---- dcsr_matrix_t ----------------------------------------------------------------
class dcsr_matrix_t:
    """Host CSR matrix read from "pp" / "mm" / "bin" (HLanc.hpp:74-392)."""

    def __init__(self, format: Optional[str] = None, filename: Optional[str] = None,
                 is_symmetric: bool = False, *, _handle=None):
        if _handle is not None:
            self._h = _handle
            return
        h = C.c_void_p()
        _check(lib().hlanc_matrix_read(format.encode(), os.fsencode(filename), int(is_symmetric), C.byref(h)),
               f"dcsr_matrix_t({format!r}, {filename!r})")
        self._h = h

    @classmethod
    def from_arrays(cls, row_ptr, col, val, ncols: int, is_symmetric: bool = False) -> "dcsr_matrix_t":
        rp = np.ascontiguousarray(row_ptr, dtype=np.int32)
        ci = np.ascontiguousarray(col, dtype=np.int32)
        va = np.ascontiguousarray(val, dtype=np.float64)
        h = C.c_void_p()
        _check(lib().hlanc_matrix_create(len(rp) - 1, int(ncols), len(ci), rp.ctypes.data, ci.ctypes.data,
                                         va.ctypes.data, int(is_symmetric), C.byref(h)), "dcsr_matrix_t")
        return cls(_handle=h)

    def _info(self):
        n, c, z, s = _i(), _i(), _i(), _i()
        _check(lib().hlanc_matrix_info(self._h, C.byref(n), C.byref(c), C.byref(z), C.byref(s)), "info")
        return n.value, c.value, z.value, bool(s.value)

    def get_num_rows(self) -> int: return self._info()[0]
    def get_num_columns(self) -> int: return self._info()[1]
    def get_nnz(self) -> int: return self._info()[2]
    def symmetric(self) -> bool: return self._info()[3]

    def _arrays(self):
        rp, ci, va = _ip(), _ip(), _dp()
        _check(lib().hlanc_matrix_arrays(self._h, C.byref(rp), C.byref(ci), C.byref(va)), "arrays")
        n, _, z, _ = self._info()
        r = np.ctypeslib.as_array(rp, shape=(n + 1,)).copy()
        c = np.ctypeslib.as_array(ci, shape=(z,)).copy() if z else np.zeros(0, np.int32)
        v = np.ctypeslib.as_array(va, shape=(z,)).copy() if z else np.zeros(0)
        return r, c, v

    def get_row_ptr(self) -> np.ndarray: return self._arrays()[0]
    def get_column_index(self) -> np.ndarray: return self._arrays()[1]
    def get_value(self) -> np.ndarray: return self._arrays()[2]

    def save_pp(self, filename): _check(lib().hlanc_matrix_save(self._h, b"pp", os.fsencode(filename)), "save_pp")
    def save_mm(self, filename): _check(lib().hlanc_matrix_save(self._h, b"mm", os.fsencode(filename)), "save_mm")
    def save_bin(self, filename): _check(lib().hlanc_matrix_save(self._h, b"bin", os.fsencode(filename)), "save_bin")

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _lib is not None:
            _lib.hlanc_matrix_destroy(h)
            self._h = None


# ---- dcsrmv_operator_gpu ---------------------------------------------------------
def _ptr(a):
    """(address, is_numpy) of a numpy array or a torch tensor."""
    if isinstance(a, np.ndarray):
        return a.ctypes.data, True
    if hasattr(a, "data_ptr"):
        return a.data_ptr(), False
    raise TypeError("expected a numpy array or a torch tensor")


class dcsrmv_operator_gpu:
    """Device CSR operator y = A x (HLanc.hpp:476-572).  Keeps the matrix's
    general CSR on device `dev`; symmetric input is expanded on construction."""

    def __init__(self, m, dev: int = 0, precision: int = HLANC_PREC_FP64):
        if isinstance(m, dcsr_matrix_t):
            rp, ci, va = m._arrays()
            n, ncols, _, sym = m._info()
        else:   # generators.CSR or any (n, ncols, row_ptr, col, val) with .symmetric optional
            rp = np.ascontiguousarray(m.row_ptr, dtype=np.int32)
            ci = np.ascontiguousarray(m.col, dtype=np.int32)
            va = np.ascontiguousarray(m.val, dtype=np.float64)
            n, ncols, sym = int(m.n), int(m.ncols), bool(getattr(m, "symmetric", False))
        h = C.c_void_p()
        _check(lib().hlanc_csr_create(dev, n, ncols, len(ci), rp.ctypes.data, ci.ctypes.data if len(ci) else None,
                                      va.ctypes.data if len(va) else None, int(sym), precision, C.byref(h)),
               "dcsrmv_operator_gpu")
        self._h, self.dev, self.n, self.ncols, self.precision = h, dev, n, ncols, precision
        self._m = m

    @property
    def handle(self):
        return self._h

    def nnz_general(self) -> int:
        z = C.c_longlong()
        _check(lib().hlanc_csr_info(self._h, None, None, None, C.byref(z), None), "info")
        return z.value

    def __call__(self, x, y) -> None:
        """operator()(x, y): numpy (host) or torch CUDA tensors (device)."""
        px, nx = _ptr(x)
        py, ny = _ptr(y)
        if nx and (x.dtype != np.float64 or not x.flags.c_contiguous):
            raise TypeError("x must be a contiguous float64 array")
        if ny and (y.dtype != np.float64 or not y.flags.c_contiguous or not y.flags.writeable):
            raise TypeError("y must be a writable contiguous float64 array")
        _check(lib().hlanc_csr_apply(self._h, px, py), "operator()")

    def tuning(self) -> dict:
        """SpMV work units chosen for this matrix (hlanc_csr_tuning)."""
        r, l4, l8 = _i(), _i(), _i()
        ud, uc = C.c_double(), C.c_double()
        _check(lib().hlanc_csr_tuning(self._h, C.byref(r), C.byref(l4), C.byref(l8), C.byref(ud), C.byref(uc)),
               "tuning")
        return {"rows_per_unit": r.value, "lanes4_mean": l4.value, "lanes8_mean": l8.value,
                "us_default": ud.value, "us_chosen": uc.value}

    def spmv_async(self, x_ptr: int, y_ptr: int, stream: int = 0) -> None:
        _check(lib().hlanc_csr_spmv_async(self._h, x_ptr, y_ptr, stream or None), "spmv_async")

    def close(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.hlanc_csr_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()


# ---- ds_solver_gpu -------------------------------------------------------------------
def ds_solver_gpu(n: int, nev: int, ncv: int, values: np.ndarray, vectors: np.ndarray, ldv: int,
                  dspmv_operator, dev: int = 0, *, opts_=None, stats: Optional[dict] = None) -> int:
    """ds_solver_gpu(n, nev, ncv, values, vectors, ldv, op, dev) (HLanc.hpp:1868-1872).

    values: float64 array of >= ncv entries; vectors: float64 array with ldv*ncv
    entries, column-major (a Fortran (ldv, ncv) array or a flat buffer).  The
    operator is a dcsrmv_operator_gpu (device-resident solve) or any callable
    op(x, y) on host float64 vectors of length n.  Returns 0 on success and 1
    when fewer than nev Ritz values converged, like the reference."""
    if values.dtype != np.float64 or values.size < ncv or not values.flags.writeable:
        raise TypeError("values must be a writable float64 array of >= ncv entries")
    if vectors.dtype != np.float64 or vectors.size < ldv * ncv or not (vectors.flags.f_contiguous or vectors.ndim == 1):
        raise TypeError("vectors must be a column-major float64 array of >= ldv*ncv entries")
    o, keep = opts_ if opts_ is not None else opts()
    st = Stats()
    cb = HOST_OP()
    csr = None
    err = []
    if isinstance(dspmv_operator, dcsrmv_operator_gpu):
        csr = dspmv_operator.handle
    else:
        def _cb(_ctx, xp, yp):
            try:
                x = np.ctypeslib.as_array(xp, shape=(n,))
                y = np.ctypeslib.as_array(yp, shape=(n,))
                dspmv_operator(x, y)
                return 0
            except BaseException as e:  # noqa: BLE001 - reported after the call
                err.append(e)
                return 1
        cb = HOST_OP(_cb)
    rc = lib().hlanc_solve(dev, n, nev, ncv, values.ctypes.data, vectors.ctypes.data, ldv, csr, cb, None,
                           C.byref(o), C.byref(st))
    if err:
        raise err[0]
    if stats is not None:
        stats.update(st.as_dict())
    if rc not in (HLANC_OK, HLANC_NOT_CONVERGED):
        raise HLancError(rc, "ds_solver_gpu")
    return rc


def solve(op, nev: int, ncv: int, dev: int = 0, **kw):
    """Convenience: returns (rc, values[:nconv], vectors (n x ncv, Fortran), stats)."""
    n = op.n if isinstance(op, dcsrmv_operator_gpu) else kw.pop("n")
    values = np.zeros(ncv)
    vectors = np.zeros((n, ncv), order="F")
    st: dict = {}
    rc = ds_solver_gpu(n, nev, ncv, values, vectors, n, op, dev, opts_=opts(**kw), stats=st)
    return rc, values[:max(st.get("nconv", 0), 0)] if rc == 0 else values, vectors, st


def solve_device(op: dcsrmv_operator_gpu, nev: int, ncv: int, values_ptr: int, vectors_ptr: int, ldv: int,
                 dev: int = 0, **kw) -> dict:
    """Solve with device-resident outputs (pointers on `dev`); returns stats."""
    o, keep = opts(**kw)
    st = Stats()
    rc = lib().hlanc_solve_device(dev, op.n, nev, ncv, values_ptr, vectors_ptr, ldv, op.handle, C.byref(o),
                                  C.byref(st))
    if rc not in (HLANC_OK, HLANC_NOT_CONVERGED):
        raise HLancError(rc, "hlanc_solve_device")
    d = st.as_dict()
    d["rc"] = rc
    return d


def residuals_device(op: dcsrmv_operator_gpu, k: int, values_ptr: int, vectors_ptr: int, ldv: int):
    """||A v_i - lambda_i v_i|| and verify_eigs' rdiff for k device pairs."""
    res = np.zeros(k)
    rd = np.zeros(k)
    _check(lib().hlanc_residuals_device(op.handle, k, values_ptr, vectors_ptr, ldv, res.ctypes.data,
                                        rd.ctypes.data), "residuals")
    return res, rd


def residuals(op: dcsrmv_operator_gpu, values: np.ndarray, vectors: np.ndarray):
    """||A v_i - lambda_i v_i|| and verify_eigs' r-diff for host pairs
    (values[k], vectors n x k), computed on the device."""
    vals = np.ascontiguousarray(values, dtype=np.float64)
    vecs = np.asfortranarray(vectors, dtype=np.float64)
    k = vals.shape[0]
    res = np.zeros(k)
    rd = np.zeros(k)
    _check(lib().hlanc_residuals_host(op.handle, k, vals.ctypes.data, vecs.ctypes.data, vecs.shape[0],
                                      res.ctypes.data, rd.ctypes.data), "residuals")
    return res, rd


def write_eigs(filename: str, values: np.ndarray, vectors: np.ndarray) -> None:
    """Eigenpair text file of the reference demo (demo/HLanc_solver_gpu.cu:57-66)."""
    vals = np.ascontiguousarray(values, dtype=np.float64)
    vecs = np.asfortranarray(vectors, dtype=np.float64)
    n = vecs.shape[0]
    _check(lib().hlanc_eigs_write(filename.encode(), vals.shape[0], n, vals.ctypes.data, vecs.ctypes.data,
                                  max(n, 1)), "eigs write")


def read_eigs(filename: str):
    """(values[nev], vectors n x nev) from an eigenpair text file (demo/verify_eigs.cu:8-44)."""
    nev, n = _i(), _i()
    _check(lib().hlanc_eigs_info(filename.encode(), C.byref(nev), C.byref(n)), "eigs info")
    vals = np.zeros(nev.value)
    vecs = np.zeros((n.value, nev.value), order="F")
    _check(lib().hlanc_eigs_read(filename.encode(), vals.ctypes.data, vecs.ctypes.data, max(n.value, 1)),
           "eigs read")
    return vals, vecs


def kernel_launches() -> int:
    return int(lib().hlanc_kernel_launches())


def kernel_launches_of(kind: int) -> int:
    """Launches since load of one kernel variant (KL_*)."""
    return int(lib().hlanc_kernel_launches_of(kind))


def variant_counts() -> dict:
    names = ("all", "proj_hybrid", "proj_fp64", "apply_shadow", "apply_fp64", "basis_tc", "basis_fp64", "cycle",
             "ritz_tc", "ritz_fp64")
    return {nm: kernel_launches_of(i) for i, nm in enumerate(names)}


def fp64_peak_tflops(dev: int = 0) -> float:
    """Measured FP64 FMA throughput of the device (TFLOP/s)."""
    t = C.c_double()
    _check(lib().hlanc_diag_fp64_tflops(dev, C.byref(t)), "fp64 probe")
    return t.value


def cgs_kernel_ms(n: int, c: int, cgs: int = HLANC_CGS_HYBRID, reps: int = 10, dev: int = 0) -> dict:
    """The CGS kernels alone on a synthetic n x c basis: mean ms per launch of
    a first-pass projection, a second-pass projection and an update."""
    ms = (C.c_double * 3)()
    _check(lib().hlanc_diag_cgs(dev, n, c, cgs, reps, ms), "cgs probe")
    return {"proj_pass1": ms[0], "proj": ms[1], "apply": ms[2]}


def last_profile() -> dict:
    """Per-kernel-class timing of the last solve run with profile=True."""
    p = Profile()
    _check(lib().hlanc_last_profile(C.byref(p)), "last_profile")
    return p.as_dict()


# ---- batched solves ------------------------------------------------------------------
class Batch:
    """Many independent solves advanced by one launch sequence per restart
    cycle (hlanc_batch_*).  Outputs are device buffers (torch tensors)."""

    def __init__(self, ops, nev, ncv, dev: int = 0, **kw):
        self.ops = list(ops)
        k = len(self.ops)
        self.nev = np.ascontiguousarray(np.broadcast_to(np.asarray(nev, dtype=np.int32), (k,)))
        self.ncv = np.ascontiguousarray(np.broadcast_to(np.asarray(ncv, dtype=np.int32), (k,)))
        self._o, self._keep = opts(**kw)
        handles = (C.c_void_p * k)(*[o.handle.value if hasattr(o.handle, "value") else o.handle for o in self.ops])
        h = C.c_void_p()
        _check(lib().hlanc_batch_create(dev, k, handles, self.nev.ctypes.data, self.ncv.ctypes.data,
                                        C.byref(self._o), C.byref(h)), "hlanc_batch_create")
        self._h, self.dev = h, dev

    def run(self, values_ptrs, vectors_ptrs):
        k = len(self.ops)
        vp = (C.c_void_p * k)(*values_ptrs)
        xp = (C.c_void_p * k)(*vectors_ptrs)
        status = np.zeros(k, dtype=np.int32)
        st = Stats()
        rc = lib().hlanc_batch_run(self._h, vp, xp, status.ctypes.data, C.byref(st))
        if rc not in (HLANC_OK, HLANC_NOT_CONVERGED):
            raise HLancError(rc, "hlanc_batch_run")
        d = st.as_dict()
        d["rc"] = rc
        return status, d

    def close(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.hlanc_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()


# ---- serving ---------------------------------------------------------------------------
class Server:
    """Continuous batching of eigen-solves (hlanc_server_*): requests are
    admitted by slot count and device-memory budget, every resident solve
    advances one restart cycle per step(), finished solves are retired.
    The residents are spread over `lanes` streams (0 = the library default)."""

    def __init__(self, mem_budget_bytes: int, max_slots: int, dev: int = 0, lanes: int = 0):
        so = ServerOpts(mem_budget_bytes, max_slots, dev, lanes)
        h = C.c_void_p()
        _check(lib().hlanc_server_create(C.byref(so), C.byref(h)), "hlanc_server_create")
        self._h, self.dev = h, dev
        self._req = {}

    def submit(self, op: dcsrmv_operator_gpu, nev: int, ncv: int, **kw) -> int:
        o, keep = opts(**kw)
        rid = C.c_longlong()
        _check(lib().hlanc_server_submit(self._h, op.handle, nev, ncv, C.byref(o), C.byref(rid)), "submit")
        self._req[rid.value] = (op.n, nev, ncv)
        return rid.value

    def step(self):
        a, p = _i(), _i()
        _check(lib().hlanc_server_step(self._h, C.byref(a), C.byref(p)), "hlanc_server_step")
        return a.value, p.value

    def poll(self, rid: int):
        n, nev, ncv = self._req[rid]
        done, status = _i(), _i()
        _check(lib().hlanc_server_poll(self._h, rid, C.byref(done), C.byref(status), None, None, None), "poll")
        if not done.value:
            return None
        values = np.zeros(ncv)
        vectors = np.zeros((n, ncv), order="F")
        st = Stats()
        _check(lib().hlanc_server_poll(self._h, rid, C.byref(done), C.byref(status), values.ctypes.data,
                                       vectors.ctypes.data, C.byref(st)), "poll")
        if not done.value:
            return None
        return status.value, values, vectors, st.as_dict()

    def cancel(self, rid: int) -> None:
        _check(lib().hlanc_server_cancel(self._h, rid), "cancel")

    def stats(self) -> dict:
        st = ServerStats()
        _check(lib().hlanc_server_stats(self._h, C.byref(st)), "hlanc_server_stats")
        return st.as_dict()

    def close(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.hlanc_server_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()
