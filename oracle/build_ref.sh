#!/usr/bin/env bash
# Build the oracle libraries (test infrastructure only).
#
#   oracle/_build/liboracle_sim.so  — the CPU restatement (oracle/oracle_sim.cpp);
#                                     built everywhere, including the GPU host.
#   oracle/_ref/libref_sim.so       — the reference engine itself, compiled from
#                                     ProjectQ's own header simulator.hpp where it
#                                     lies in the reference tree; built only when
#                                     that tree is present (REFERENCE_ROOT).
#
# The reference flags follow its setup.py: -O3 -fopenmp -std=c++17 and, on
# x86, -march=native -DINTRIN (AVX2 kernels); elsewhere the portable
# nointrin kernels.
set -euo pipefail
here="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
mkdir -p "$here/_build"
g++ -O3 -std=c++17 -fopenmp -fPIC -shared -ffp-contract=fast \
    "$here/oracle_sim.cpp" -o "$here/_build/liboracle_sim.so.tmp"
mv "$here/_build/liboracle_sim.so.tmp" "$here/_build/liboracle_sim.so"

ref_root="${REFERENCE_ROOT:-/root/reference}"
hdr="$ref_root/projectq/backends/_sim/_cppkernels"
if [[ -f "$hdr/simulator.hpp" ]]; then
  mkdir -p "$here/_ref"
  arch_flags=()
  if [[ "$(uname -m)" == "x86_64" ]]; then arch_flags=(-march=native -DINTRIN); fi
  g++ -O3 -std=c++17 -fopenmp -fPIC -shared "${arch_flags[@]}" -I"$hdr" \
      "$here/ref_driver.cpp" -o "$here/_ref/libref_sim.so.tmp"
  mv "$here/_ref/libref_sim.so.tmp" "$here/_ref/libref_sim.so"
fi
