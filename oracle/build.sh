#!/usr/bin/env bash
# Builds the CPU oracle (test infrastructure) into oracle/_build/liboracle.so.
# -ffp-contract=off keeps x86-64 and aarch64 results identical (no fused multiply-add contraction).
set -euo pipefail
here="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
mkdir -p "$here/_build"
g++ -O2 -std=c++17 -ffp-contract=off -fopenmp -fPIC -shared -o "$here/_build/liboracle.so.tmp" "$here/oracle.cpp"
mv "$here/_build/liboracle.so.tmp" "$here/_build/liboracle.so"
