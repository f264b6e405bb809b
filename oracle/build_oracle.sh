#!/usr/bin/env bash
# Builds oracle/libsvo_oracle.so, the CPU restatement used as the parity
# checker and the timed CPU baseline. TEST INFRASTRUCTURE ONLY.
# Strict IEEE binary32 (-ffp-contract=off), no target-specific flags, so the
# same source gives the same results on x86-64 and aarch64 hosts.
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
g++ -std=c++17 -O3 -ffp-contract=off -fno-fast-math -fopenmp -fPIC -shared -Wall -Wno-unused-function \
    -o "$HERE/libsvo_oracle.so.tmp" "$HERE/svo_oracle.cpp"
mv "$HERE/libsvo_oracle.so.tmp" "$HERE/libsvo_oracle.so"
echo "build_oracle: built $HERE/libsvo_oracle.so"
