#!/bin/sh
# Build the oracle's C checker library (test infrastructure only).
# -ffp-contract=off: every fused multiply-add in rng_oracle.c is an explicit fmaf().
set -e
here="$(cd "$(dirname "$0")" && pwd)"
mkdir -p "$here/_build"
${CC:-gcc} -O2 -ffp-contract=off -fPIC -shared -std=c11 \
    -o "$here/_build/liboracle_rng.so" "$here/rng_oracle.c" -lm
