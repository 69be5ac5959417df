#!/usr/bin/env bash
# Build the oracle libraries (test and baseline infrastructure only).
#
#   oracle/_build/liboracle_sim.so  — the CPU restatement (oracle/oracle_sim.cpp);
#                                     built everywhere.
#   oracle/_ref/libref_sim.so       — the reference engine itself, compiled from
#                                     ProjectQ's own header simulator.hpp where it
#                                     lies in the reference tree, with the flags the
#                                     golden fixtures were made with (-O3; on x86
#                                     -march=native -DINTRIN, the AVX kernels).
#   oracle/_ref/libref_sim_setup.so — the same engine with the flags ProjectQ's
#                                     setup.py gives it (python's -DNDEBUG -O2,
#                                     -fopenmp, -ffast-math, -std=c++17; on x86
#                                     -march=native -DINTRIN, elsewhere the portable
#                                     nointrin kernels, setup.py:535-571): the CPU
#                                     baseline that bench.py times.
#
# The reference tree is REFERENCE_ROOT, by default baseline/_ref (the reference
# installed next to this repository with pip, which carries the C++ headers);
# without it only the restatement is built.
set -euo pipefail
here="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
mkdir -p "$here/_build"
g++ -O3 -std=c++17 -fopenmp -fPIC -shared -ffp-contract=fast \
    "$here/oracle_sim.cpp" -o "$here/_build/liboracle_sim.so.tmp" &
pids=($!)

ref_root="${REFERENCE_ROOT:-$here/../baseline/_ref}"
hdr="$ref_root/projectq/backends/_sim/_cppkernels"
if [[ -f "$hdr/simulator.hpp" ]]; then
  mkdir -p "$here/_ref"
  arch_flags=()
  if [[ "$(uname -m)" == "x86_64" ]]; then arch_flags=(-march=native -DINTRIN); fi
  g++ -O3 -std=c++17 -fopenmp -fPIC -shared "${arch_flags[@]}" -I"$hdr" \
      "$here/ref_driver.cpp" -o "$here/_ref/libref_sim.so.tmp" &
  pids+=($!)
  g++ -DNDEBUG -O2 -std=c++17 -fopenmp -ffast-math -fPIC -shared "${arch_flags[@]}" -I"$hdr" \
      "$here/ref_driver.cpp" -o "$here/_ref/libref_sim_setup.so.tmp" &
  pids+=($!)
fi
for p in "${pids[@]}"; do wait "$p"; done
mv "$here/_build/liboracle_sim.so.tmp" "$here/_build/liboracle_sim.so"
if [[ -f "$hdr/simulator.hpp" ]]; then
  mv "$here/_ref/libref_sim.so.tmp" "$here/_ref/libref_sim.so"
  mv "$here/_ref/libref_sim_setup.so.tmp" "$here/_ref/libref_sim_setup.so"
fi
