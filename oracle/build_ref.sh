#!/bin/sh
# Builds pyquafu's qfvm CPU module (src/qfvm/qfvm.cpp, unmodified, read where it
# lies in the reference tree) into oracle/_ref/ for parity checks.  Eigen and
# pybind11/eigen.h come from the stand-ins in oracle/shim/.  Flags follow the
# reference CMakeLists.txt:66-76 (Release -O3; on x86_64 -mfma -mavx2
# -ffast-math -DUSE_SIMD; OpenMP with ENABLE_OPENMP).
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${QFVM_REFERENCE_ROOT:-/root/reference}
[ -f "$REF/src/qfvm/qfvm.cpp" ] || { echo "reference sources not found under $REF" >&2; exit 3; }
PY=${PYTHON:-python3}
PYBIND=$($PY -c "import pybind11; print(pybind11.get_include())")
PYINC=$($PY -c "import sysconfig; print(sysconfig.get_paths()['include'])")
EXT=$($PY -c "import sysconfig; print(sysconfig.get_config_var('EXT_SUFFIX'))")
case "$(uname -m)" in
  x86_64|amd64) SIMD="-mfma -mavx2 -ffast-math -DUSE_SIMD" ;;
  *) SIMD="" ;;
esac
mkdir -p "$HERE/_ref"
# where the sources were read from, for oracle/refload.py
echo "$REF" > "$HERE/_ref/reference_root"
OUT="$HERE/_ref/qfvm$EXT"
if [ -f "$OUT" ] && [ "$OUT" -nt "$REF/src/qfvm/qfvm.cpp" ] && [ "${1:-}" != "--force" ]; then
  echo "$OUT"
  exit 0
fi
g++ -std=c++20 -O3 -shared -fPIC -fvisibility=hidden -fopenmp -DENABLE_OPENMP $SIMD \
    -I"$HERE/shim" -I"$PYBIND" -I"$PYINC" -I"$REF/src/qfvm" -I"$REF/src/qfvm_clifford" \
    "$REF/src/qfvm/qfvm.cpp" -o "$HERE/_ref/qfvm$EXT"
echo "$HERE/_ref/qfvm$EXT"
