#!/usr/bin/env bash
# Builds oracle/_ref/libptgpu_ref.so: the reference's own CLBVH.cpp, KDTree.cpp,
# displayfunc.cpp, BVH.cl, rendering_kernel.cl and geomfunc.h compiled on the
# CPU (TEST INFRASTRUCTURE: it pins the oracle restatement).  Sources are read
# where they lie in the reference tree; only BVH.cl is copied, into
# oracle/_ref/gen/, with one guard added to its split-search loop (the loop
# never reaches t = 0 and ends in an integer division by zero on the CPU).
# Everything written goes under oracle/_ref/, which git ignores.
set -euo pipefail
# the reference tree is named only by PTGPU_REFERENCE_DIR
REF=${PTGPU_REFERENCE_DIR:-}
if [ -z "$REF" ]; then echo "PTGPU_REFERENCE_DIR is not set: the reference build is skipped" >&2; exit 3; fi
HERE=$(cd "$(dirname "$0")" && pwd)
OUT=$(cd "$HERE/.." && pwd)/_ref
if [ ! -f "$REF/include/BVH.cl" ]; then echo "reference tree not found at $REF" >&2; exit 3; fi
SHIM=$OUT/shim; GEN=$OUT/gen; OBJ=$OUT/obj
mkdir -p "$SHIM" "$GEN" "$OBJ"
# the reference includes headers as "include\\x.h" and "CL\\cl.h": file names
# with a literal double backslash resolve through these links
ln -sfn "$REF/include" "$SHIM/include"
for h in geom.h BVHNodeGPU.h KDNodeGPU.h CLBVH.h KDTree.h AccelCommon.h native-lib.h ply.h; do
  ln -sfn "$REF/include/$h" "$SHIM/include\\\\$h"
done
ln -sfn "$HERE/cl_stub.h" "$SHIM/CL\\\\cl.h"
ln -sfn "$HERE/stdafx_stub.h" "$SHIM/stdafx.h"
sed 's|t = (l + (divider - 1)) / divider; t >= 1; divider \*= 2)|t = (l + (divider - 1)) / divider; t >= 1 \&\& divider < (1 << 30); divider *= 2)|' \
  "$REF/include/BVH.cl" > "$GEN/BVH.cl"
grep -q 'divider < (1 << 30)' "$GEN/BVH.cl" || { echo "BVH.cl guard not applied" >&2; exit 4; }
CXX=${CXX:-g++}
FLAGS="-O2 -ffp-contract=off -fno-fast-math -fPIC -std=c++17 -w"
$CXX $FLAGS -iquote "$SHIM" -I "$GEN" -I "$SHIM/include" -I "$HERE" -c "$HERE/ref_kernels.cpp" -o "$OBJ/ref_kernels.o" &
( cd "$SHIM" && $CXX $FLAGS -iquote . -I "$SHIM/include" -x c++ -c - -o "$OBJ/clbvh.o" < "$REF/CLBVH.cpp" ) &
( cd "$SHIM" && $CXX $FLAGS -iquote . -I "$SHIM/include" -x c++ -c - -o "$OBJ/kdtree.o" < "$REF/KDTree.cpp" ) &
( cd "$SHIM" && $CXX $FLAGS -iquote . -I "$SHIM/include" -include errno.h -x c++ -c - -o "$OBJ/displayfunc.o" < "$REF/displayfunc.cpp" ) &
( cd "$SHIM" && $CXX $FLAGS -iquote . -I "$SHIM/include" -c "$HERE/ref_glue.cpp" -o "$OBJ/ref_glue.o" ) &
for a in 0 1 2; do
  ( cd "$SHIM" && $CXX $FLAGS -fopenmp -iquote . -I "$SHIM/include" -DREF_ACCEL=$a -c "$HERE/ref_cpu.cpp" -o "$OBJ/ref_cpu$a.o" ) &
done
wait_all() { local rc=0; for j in $(jobs -p); do wait "$j" || rc=1; done; return $rc; }
wait_all
$CXX -shared -fopenmp -o "$OUT/libptgpu_ref.so" "$OBJ"/*.o -lm
echo "built $OUT/libptgpu_ref.so"
