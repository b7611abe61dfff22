#!/usr/bin/env bash
# Builds oracle/_ref/libdpref.so: the reference's own kernel sources
# (mmccraw98/dpCUDA-v2 src/particles/{base,disk,rigid_bumpy}/kernels.cu, read in
# place, never copied) compiled as host C++ through shim/, linked with
# ref_driver.cpp / ref_bumpy_driver.cpp.  TEST INFRASTRUCTURE ONLY: used to pin
# the oracle and to generate tests/golden fixtures.  Needs the reference tree,
# named by DPG_REFERENCE; exits 0 without building when that is unset or the
# tree is absent.
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF="${DPG_REFERENCE:-}"
OUT="$HERE/../_ref"
if [ -z "$REF" ] || [ ! -d "$REF/src/particles" ]; then
  echo "DPG_REFERENCE does not name the reference tree; oracle/_ref not built"
  exit 0
fi
mkdir -p "$OUT"
CXX="${CXX:-g++}"
FLAGS=(-std=c++17 -O2 -fPIC -fopenmp -ffp-contract=off -fno-fast-math -w
       -include "$HERE/shim/cuda_host_shim.h" -I "$HERE/shim" -I "$REF/include"
       -I /usr/local/cuda/include/cccl -I /usr/local/cuda/include)
objs=()
for k in base disk rigid_bumpy; do
  "$CXX" "${FLAGS[@]}" -x c++ -c "$REF/src/particles/$k/kernels.cu" -o "$OUT/ref_${k}_kernels.o" &
  objs+=("$OUT/ref_${k}_kernels.o")
done
for d in ref_driver ref_bumpy_driver; do
  if [ -f "$HERE/$d.cpp" ]; then
    "$CXX" "${FLAGS[@]}" -c "$HERE/$d.cpp" -o "$OUT/$d.o" &
    objs+=("$OUT/$d.o")
  fi
done
wait
"$CXX" -shared -fopenmp -o "$OUT/libdpref.so" "${objs[@]}"
echo "built $OUT/libdpref.so"
