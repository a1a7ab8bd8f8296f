"""CPU oracle for the HLanc IRLM path -- test infrastructure only.

Importable by the test-suite, by __graft_entry__.smoke() and by bench.py's
CPU-baseline leg, and only as the checker (or the timed CPU baseline).  The
product package ``hlanc_gb300`` never imports it.

- ``liboracle.so``: the plain-C restatement (hlanc_oracle.c), built by
  ``build()`` with gcc (OpenMP) on any host.
- ``_ref/libhlanc_ref.so``: the reference's own CPU path compiled through the
  MKL shim (build_ref.sh); it exists only where the reference sources are
  mounted, and is used to pin the restatement and write the golden fixtures.
"""
from .pyoracle import (  # noqa: F401
    build, lib, ref_lib, solve_csr, spmv, read_matrix, save_matrix, tridiag_eig,
    ref_available, ref_solve_csr, ref_spmv, ref_read, ref_save,
)
