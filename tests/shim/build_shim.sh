#!/usr/bin/env bash
# Builds the reference-side drop-in GB300Renderer (tests/shim/GB300Renderer.cu) and its test
# harness (tests/shim/shim_driver.cu) against the reference sources into
# tests/shim/_build/libgb300shim.so, linked with the reference host path (oracle/_ref/libdumbref.so,
# built by oracle/build_ref.sh) and the library (dumbray_gb300/_build/libdumbray_gb300.so).
# Flags follow oracle/build_ref.sh: the reference headers need -rdc and C++14.  Exit 3 when the
# reference build is absent.
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
ROOT="$(cd "$HERE/../.." && pwd)"
S="$ROOT/oracle/_ref/src/__source__"
REF_LIB="$ROOT/oracle/_ref/libdumbref.so"
LIB_DIR="$ROOT/dumbray_gb300/_build"
if [ ! -d "$S" ] || [ ! -f "$REF_LIB" ]; then
  echo "build_shim.sh: the reference build (oracle/build_ref.sh) is missing" >&2
  exit 3
fi
[ -f "$LIB_DIR/libdumbray_gb300.so" ] || python3 -c "import sys; sys.path.insert(0, '$ROOT'); from dumbray_gb300 import build; build.build()"
OUT="$HERE/_build"
mkdir -p "$OUT"
ARCH="${DUMBRAY_REF_ARCH:-sm_100}"
FLAGS=(-std=c++14 -O2 -rdc=true -arch="$ARCH" -w -Xcompiler -fPIC -Xcompiler -ffp-contract=off
       -I"$S" -I"$ROOT/include" -I"$ROOT/oracle" -I"$HERE")
nvcc "${FLAGS[@]}" -dc "$HERE/GB300Renderer.cu" -o "$OUT/GB300Renderer.o" &
p1=$!
nvcc "${FLAGS[@]}" -dc "$HERE/shim_driver.cu" -o "$OUT/shim_driver.o" &
p2=$!
wait $p1
wait $p2
nvcc -arch="$ARCH" -dlink "$OUT/GB300Renderer.o" "$OUT/shim_driver.o" -Xcompiler -fPIC -o "$OUT/dlink.o"
g++ -shared -Wl,--no-undefined -o "$OUT/libgb300shim.so" "$OUT/GB300Renderer.o" "$OUT/shim_driver.o" "$OUT/dlink.o" \
    -L"$ROOT/oracle/_ref" -ldumbref -L"$LIB_DIR" -ldumbray_gb300 -L/usr/local/cuda/lib64 -lcudart -lpthread \
    -Wl,-rpath,"$ROOT/oracle/_ref" -Wl,-rpath,"$LIB_DIR"
echo "built $OUT/libgb300shim.so"
