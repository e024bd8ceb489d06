#!/usr/bin/env bash
# Builds the CPU oracle (test infrastructure) into oracle/_build/libdroracle.so.
# FP contraction is off so the float restatement rounds exactly like the reference's host build
# on both x86-64 and aarch64.
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
mkdir -p "$HERE/_build"
g++ -std=c++17 -O2 -ffp-contract=off -fPIC -shared -pthread -Wall -Wno-unused-function \
    -o "$HERE/_build/libdroracle.so" "$HERE/dr_oracle.cpp"
echo "built $HERE/_build/libdroracle.so"
