#!/usr/bin/env bash
# Builds the reference DumbRay CPU path (octree cast + DumbRenderer on host threads) into
# oracle/_ref/libdumbref.so (plus its PNG writer, Images::saveBufferPNG + lodepng, and its scene-file
# loader, DumbRenderContext with the Dson parser), for use as a parity checker and as the timed CPU
# baseline.  The translation units are a subset of the reference's own Linux list
# (UBUNTU_BUILD/__MAKE__.sh); DumbRenderContext.cu is compiled through oracle/ref_dumb.cu, which
# includes it.  The window classes it links against are compiled but never called.
#
# The reference sources are read from $DUMBRAY_REFERENCE (default: the read-only checkout at
# /root/reference).  They are copied into oracle/_ref/src (git-ignored) because two portability
# patches are needed before gcc 13 / CUDA 13 accept them:
#   (1) Generic.impl.cuh: dependent member-template calls need the `template` keyword
#       (`memoryManagementModule.template use<Type>()`, `destination.template use<Type>(...)`);
#   (2) Device.cu: cudaDeviceProp fields removed in CUDA 13 (clockRate, deviceOverlap,
#       kernelExecTimeoutEnabled, computeMode, ...) are no longer printed;
#   (3) Windows.cu: the non-Windows no-op window stub defines its constructor with a `const char *`
#       name where the header declares `const wchar_t *`; the definition takes the declared type.
# Nothing else in the reference is changed.  The reference's own build script is not used.
#
# When no reference checkout is present but oracle/_ref/src already holds the patched copy
# (e.g. a machine that received this tree without the checkout), the copy is reused.
#
# Host code is compiled -O2 without fast-math and with FP contraction off, so results are the same
# on x86-64 and aarch64.
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
REF="${DUMBRAY_REFERENCE:-/root/reference}"
SRC="$OUT/src"
mkdir -p "$OUT"

if [ -d "$REF/__source__" ]; then
  rm -rf "$SRC.tmp"
  mkdir -p "$SRC.tmp"
  cp -r "$REF/__source__" "$SRC.tmp/"
  G="$SRC.tmp/__source__/DataStructures/GeneralPurpose/Generic/Generic.impl.cuh"
  sed -i 's/memoryManagementModule\.use<Type>()/memoryManagementModule.template use<Type>()/' "$G"
  sed -i 's/destination\.use<Type>(/destination.template use<Type>(/' "$G"
  D="$SRC.tmp/__source__/Namespaces/Device/Device.cu"
  sed -i -E '/properties\.(clockRate|deviceOverlap|kernelExecTimeoutEnabled|computeMode|memoryClockRate|maxTexture1DLinear|cooperativeMultiDeviceLaunch)/d' "$D"
  W="$SRC.tmp/__source__/Namespaces/Windows/Windows.cu"
  sed -i 's/^Windows::Window::Window(const char \*windowName/Windows::Window::Window(const wchar_t *windowName/' "$W"
  rm -rf "$SRC"
  mv "$SRC.tmp" "$SRC"
  # the reference's example scene (scene file + OBJ), read by the scene-file parity tests
  rm -rf "$OUT/example_scenes"
  cp -r "$REF/example_scenes" "$OUT/example_scenes"
elif [ ! -d "$SRC/__source__" ]; then
  echo "build_ref.sh: no reference checkout at $REF and no patched copy in $SRC" >&2
  exit 3
fi

S="$SRC/__source__"
TUS=(
  "$S/DataStructures/Renderers/DumbRenderer/DumbRenderer.cu"
  "$S/DataStructures/Renderers/BlockRenderer/BlockRenderer.cu"
  "$S/DataStructures/Renderers/Renderer/Renderer.cu"
  "$S/DataStructures/Renderers/BufferedRenderer/BufferedRenderer.cu"
  "$S/DataStructures/GeneralPurpose/DumbRand/DumbRand.cu"
  "$S/DataStructures/GeneralPurpose/Semaphore/Semaphore.cu"
  "$S/DataStructures/Screen/FrameBuffer/BlockBasedFrameBuffer/BlockBasedFrameBuffer.impl.cu"
  "$S/Namespaces/Device/Device.cu"
  "$S/Namespaces/Images/Images.cu"
  "$S/Namespaces/Images/lodepng.cu"
  "$S/DataStructures/DumbRenderContext/DumbRenderContextRegistry.cu"
  "$S/DataStructures/Objects/Components/DumbStructs.cu"
  "$S/DataStructures/Renderers/BufferedRenderProcess/BufferedRenderProcess.cu"
  "$S/DataStructures/Screen/BufferedWindow/BufferedWindow.cu"
  "$S/DataStructures/Screen/Window/WindowsWindow.cu"
  "$S/Namespaces/Windows/Windows.cu"
  "$S/Namespaces/Dson/Dson.cu"
  "$S/Namespaces/TextParser/ByteSet.cu"
  "$S/Namespaces/TextParser/Error.cu"
  "$S/Namespaces/TextParser/ParserNetwork.cu"
  "$S/Namespaces/TextParser/RecursiveParser.cu"
  "$HERE/ref_driver.cu"
  "$HERE/ref_dumb.cu"
)
ARCH="${DUMBRAY_REF_ARCH:-sm_100}"
OBJ="$OUT/obj"
mkdir -p "$OBJ"
FLAGS=(-std=c++14 -O2 -rdc=true -arch="$ARCH" -w -Xcompiler -fPIC -Xcompiler -ffp-contract=off -I"$S")
pids=()
objs=()
for tu in "${TUS[@]}"; do
  o="$OBJ/$(basename "$tu" .cu).o"
  objs+=("$o")
  nvcc "${FLAGS[@]}" -dc "$tu" -o "$o" &
  pids+=($!)
done
rc=0
for p in "${pids[@]}"; do wait "$p" || rc=1; done
[ $rc -eq 0 ] || { echo "build_ref.sh: compile failed" >&2; exit 1; }
nvcc -arch="$ARCH" -dlink "${objs[@]}" -Xcompiler -fPIC -o "$OBJ/dlink.o"
g++ -shared -Wl,--no-undefined -o "$OUT/libdumbref.so" "${objs[@]}" "$OBJ/dlink.o" -L/usr/local/cuda/lib64 -lcudart -lpthread
echo "built $OUT/libdumbref.so"
