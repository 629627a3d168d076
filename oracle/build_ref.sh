#!/bin/sh
# Test infrastructure only: builds the reference's own C++ window kernel
# (src/lrft_cpp.cpp of albert-hzbn/LResDFT, compiled unchanged from where it lies)
# into oracle/_ref/, so that the golden-vector generator can run the reference
# LRFTLCAOCpp path.  The reference expects a system OpenBLAS (-lopenblas); this
# image has none, so the LAPACK symbols are mapped onto the copies exported by
# scipy's bundled OpenBLAS (exported names only, nothing is disassembled).
#
# Usage: sh oracle/build_ref.sh REFERENCE_ROOT   (or LRES_REFERENCE_ROOT in the environment)
# Needs pybind11 (present in the x86 build container only); on machines without
# it or without the reference tree the script exits 0 and builds nothing.
set -e
REF=${1:-${LRES_REFERENCE_ROOT:-}}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
if [ -z "$REF" ]; then
    echo "build_ref: no reference root given (argument or LRES_REFERENCE_ROOT); skipped"
    exit 0
fi
if [ ! -f "$REF/src/lrft_cpp.cpp" ]; then
    echo "build_ref: no reference tree at $REF; skipped"
    exit 0
fi
if ! python3 -c "import pybind11" 2>/dev/null; then
    echo "build_ref: pybind11 not importable; skipped"
    exit 0
fi
mkdir -p "$OUT"
SCIPY_LIBS=$(python3 -c 'import scipy,os;print(os.path.realpath(os.path.join(os.path.dirname(scipy.__file__),"..","scipy.libs")))')
BLAS=$(ls "$SCIPY_LIBS"/libscipy_openblas*.so | head -1)
SUF=$(python3-config --extension-suffix)
g++ -O3 -fopenmp -shared -fPIC -std=c++17 \
    -Ddsygvx_=scipy_dsygvx_ -Ddsygvd_=scipy_dsygvd_ -Ddpotrf_=scipy_dpotrf_ \
    -Ddsygst_=scipy_dsygst_ -Ddsyevr_=scipy_dsyevr_ -Ddtrsm_=scipy_dtrsm_ \
    -Ddsyrk_=scipy_dsyrk_ -Dopenblas_set_num_threads=scipy_openblas_set_num_threads \
    $(python3 -m pybind11 --includes) "$REF/src/lrft_cpp.cpp" \
    -o "$OUT/_lrft_cpp$SUF" "$BLAS" -Wl,-rpath,"$SCIPY_LIBS"
echo "build_ref: built $OUT/_lrft_cpp$SUF"
