#!/usr/bin/env bash
# Test infrastructure only.  Compiles the reference's own CPU library
# (deepmodeling/deepmd-kit source/lib/src/*.cc, read in place from the
# read-only reference checkout) plus oracle/ref_shim.cc into
# oracle/_ref/libdeepmd_ref.so.  No reference source is copied.  Used to pin
# the restated oracle and to generate tests/golden fixtures; never shipped.
set -euo pipefail
REF=${DPGB_REFERENCE:-/root/reference}
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
if [ ! -d "$REF/source/lib/src" ]; then
  echo "build_ref: reference sources not present at $REF; skipping" >&2
  exit 0
fi
mkdir -p "$OUT/obj"
SRCS="env_mat fmt_nlist prod_env_mat prod_force prod_virial prod_force_grad prod_virial_grad tabulate neighbor_list coord region utilities SimulationRegion"
pids=()
for f in $SRCS; do
  src=$(ls "$REF/source/lib/src/$f".c* | head -1)
  g++ -O2 -fPIC -fopenmp -std=c++17 -I "$REF/source/lib/include" -c "$src" -o "$OUT/obj/$f.o" &
  pids+=($!)
done
g++ -O2 -fPIC -fopenmp -std=c++17 -I "$REF/source/lib/include" -c "$HERE/ref_shim.cc" -o "$OUT/obj/ref_shim.o" &
pids+=($!)
for p in "${pids[@]}"; do wait "$p"; done
g++ -shared -fopenmp -o "$OUT/libdeepmd_ref.so" "$OUT"/obj/*.o
echo "build_ref: wrote $OUT/libdeepmd_ref.so"

# The reference's PyTorch op library (source/op/pt/tabulate_multi_device.cc),
# CPU build, so the reference model can run its compressed form here.
TORCH_DIR=$(python3 -c "import os, torch; print(os.path.dirname(torch.__file__))")
if [ ! -f "$OUT/libdeepmd_op_pt.so" ] || [ "$REF/source/op/pt/tabulate_multi_device.cc" -nt "$OUT/libdeepmd_op_pt.so" ]; then
  g++ -O2 -fPIC -std=c++17 -D_GLIBCXX_USE_CXX11_ABI=1 -I "$REF/source/lib/include" \
    -I "$TORCH_DIR/include" -I "$TORCH_DIR/include/torch/csrc/api/include" \
    -shared -o "$OUT/libdeepmd_op_pt.so" "$REF/source/op/pt/tabulate_multi_device.cc" \
    "$OUT/obj/tabulate.o" -L "$TORCH_DIR/lib" -ltorch -ltorch_cpu -lc10 -fopenmp \
    -Wl,-rpath,"$TORCH_DIR/lib"
  echo "build_ref: wrote $OUT/libdeepmd_op_pt.so"
fi
