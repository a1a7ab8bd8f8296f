#!/bin/sh
# Build the reference's own CPU solver (HLanc.hpp, unmodified) into
# oracle/_ref/libhlanc_ref.so.  Checker only: used in the development
# container to pin the oracle restatement and to write tests/golden/.
# Needs the reference sources (HLANC_REFERENCE, else a directory named
# reference beside the repository),
# nvcc (the header defines two __global__ kernels) and scipy's bundled
# OpenBLAS as the MKL stand-in (oracle/ref_shim/mkl.h).
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${HLANC_REFERENCE:-$(cd "$HERE/../.." && pwd)/reference}
if [ ! -f "$REF/HLanc.hpp" ]; then
    echo "build_ref: reference sources not found at $REF; skipping" >&2
    exit 0
fi
LIBDIR=$(python3 -c "import scipy, os; print(os.path.join(os.path.dirname(scipy.__file__), '..', 'scipy.libs'))")
OPENBLAS=$(ls "$LIBDIR" | grep -m1 '^libscipy_openblas.*\.so$' || true)
if [ -z "$OPENBLAS" ]; then
    echo "build_ref: scipy-bundled OpenBLAS not found; skipping" >&2
    exit 0
fi
LIBDIR=$(cd "$LIBDIR" && pwd)
mkdir -p "$HERE/_ref"
nvcc -O2 -std=c++17 -w -Xcompiler -fPIC -shared \
    -I "$HERE/ref_shim" -I "$REF" \
    "$HERE/ref_shim/ref_wrap.cu" -o "$HERE/_ref/libhlanc_ref.so" \
    -L "$LIBDIR" -l:"$OPENBLAS" -Xlinker -rpath,"$LIBDIR" -lcublas -lcusparse
echo "build_ref: built $HERE/_ref/libhlanc_ref.so"
