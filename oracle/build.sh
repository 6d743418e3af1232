#!/bin/sh
# Builds the CPU oracle (test infrastructure) into oracle/_build/liboracle.so.
set -e
HERE="$(cd "$(dirname "$0")" && pwd)"
mkdir -p "$HERE/_build"
${CC:-gcc} -O2 -std=c11 -fPIC -shared -fopenmp -ffp-contract=off -fno-fast-math \
  -o "$HERE/_build/liboracle.so" "$HERE/oracle.c" -lm
