#!/bin/sh
# Compile the reference's own demo programs that use only the GPU API
# (demo/matrix_convertor.cu, demo/verify_eigs.cu, demo/HLanc_solver_gpu.cu),
# unmodified, against this repository's include/HLanc.hpp and libhlanc_gb300.
# The demos include "../HLanc.hpp"; they are built in a scratch tree ($1)
# whose HLanc.hpp includes this repository's header.  Exit 3 when the
# reference sources are absent (HLANC_REFERENCE, else a directory named
# reference beside the repository).
set -e
OUT=$1
HERE=$(cd "$(dirname "$0")/../.." && pwd)
REF=${HLANC_REFERENCE:-$(dirname "$HERE")/reference}
[ -d "$REF/demo" ] || { echo "reference demos not found at $REF" >&2; exit 3; }
mkdir -p "$OUT/demo"
echo "#include \"$HERE/include/HLanc.hpp\"" > "$OUT/HLanc.hpp"
for f in matrix_convertor verify_eigs HLanc_solver_gpu; do
    cp "$REF/demo/$f.cu" "$OUT/demo/$f.cu"
    (cd "$OUT/demo" && nvcc -std=c++17 -O2 -gencode arch=compute_103a,code=sm_103a -I "$HERE/include" \
        "$f.cu" -o "$OUT/$f" -L "$HERE/hlanc_gb300" -lhlanc_gb300 -Xlinker "-rpath=$HERE/hlanc_gb300")
done
