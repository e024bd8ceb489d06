#!/usr/bin/env bash
# Builds the reference-side drop-in GB300Renderer (tests/shim/GB300Renderer.cu) and its test
# harness (tests/shim/shim_driver.cu) against the reference sources into
# tests/shim/_build/libgb300shim.so, linked with the library (dumbray_gb300/_build/libdumbray_gb300.so).
#
# The shared object also holds the reference's own objects as oracle/build_ref.sh compiled them
# (oracle/_ref/obj: DumbRenderer, BlockRenderer, the frame buffers, the scene records of
# ref_driver.cu, ...), as one binary, the way the shim sits inside a DumbRay build: the shim tells
# shaders, lenses and lights apart by their function-pack pointers, which are only comparable
# within one binary.  Flags follow oracle/build_ref.sh (the reference headers need -rdc and C++14).
# Exit 3 when the reference build is absent.
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
REF_OBJS=()
for o in "$ROOT"/oracle/_ref/obj/*.o; do
  [ "$(basename "$o")" = dlink.o ] || REF_OBJS+=("$o")
done
OBJS=("$OUT/GB300Renderer.o" "$OUT/shim_driver.o" "${REF_OBJS[@]}")
nvcc -arch="$ARCH" -dlink "${OBJS[@]}" -Xcompiler -fPIC -o "$OUT/dlink.o"
g++ -shared -Wl,--no-undefined -o "$OUT/libgb300shim.so" "${OBJS[@]}" "$OUT/dlink.o" \
    -L"$LIB_DIR" -ldumbray_gb300 -L/usr/local/cuda/lib64 -lcudart -lpthread -Wl,-rpath,"$LIB_DIR"
echo "built $OUT/libgb300shim.so"
