#!/usr/bin/env bash
# Builds the CPU oracle oracle/_build/liboracle.so (test infrastructure only).
# IEEE binary32 in source order: no FMA contraction, no fast-math.
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
mkdir -p "$HERE/_build"
gcc -std=gnu11 -O2 -fPIC -shared -fopenmp -ffp-contract=off -fno-fast-math -Wall -Wno-unused-function \
    -o "$HERE/_build/liboracle.so" "$HERE"/oracle_*.c -lm
echo "built $HERE/_build/liboracle.so"
