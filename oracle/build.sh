#!/bin/sh
# Builds the oracle (test infrastructure only) into oracle/_build/.
#
# liboracle.so: the parity checker.  Plain g++ -O3 with no -march/-mcpu flag,
# so that the same recipe gives the same results on x86_64 and aarch64.
# liboracle_native.so: the same source tuned for the host CPU (-O3 -mcpu=native
# on aarch64, -O3 -march=native on x86_64: FMA, SVE2/AVX as the CPU has them),
# used only to time the CPU baseline.  Its flags are written beside it.
set -e
here="$(cd "$(dirname "$0")" && pwd)"
mkdir -p "$here/_build"
common="-std=c++17 -fopenmp -fPIC -shared -Wall -Wno-unused-function"
case "$(uname -m)" in
  aarch64|arm64) tune="-mcpu=native" ;;
  *) tune="-march=native" ;;
esac
# both builds in parallel; a failing native build only drops the tuned library
( if g++ -O3 $tune $common -o "$here/_build/liboracle_native.so" "$here/trixi_oracle.cpp" \
       2>/dev/null; then
    echo "g++ -O3 $tune -fopenmp" > "$here/_build/liboracle_native.flags"
  else
    rm -f "$here/_build/liboracle_native.so" "$here/_build/liboracle_native.flags"
  fi ) &
native=$!
g++ -O3 $common -o "$here/_build/liboracle.so" "$here/trixi_oracle.cpp"
wait $native || true
