#!/bin/sh
# Builds the oracle (test infrastructure only) into oracle/_build/.
# Plain g++; no -march flags so that the same recipe works on x86_64 and aarch64.
set -e
here="$(cd "$(dirname "$0")" && pwd)"
mkdir -p "$here/_build"
g++ -O3 -std=c++17 -fopenmp -fPIC -shared -Wall -Wno-unused-function \
    -o "$here/_build/liboracle.so" "$here/trixi_oracle.cpp"
