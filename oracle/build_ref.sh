#!/usr/bin/env bash
# Test infrastructure only.  Compiles the reference's own CPU library
# (deepmodeling/deepmd-kit source/lib/src/*.cc, read in place from the
# read-only reference checkout) plus oracle/ref_shim.cc into
# oracle/_ref/libdeepmd_ref.so.  No reference source is copied.  Used to pin
# the restated oracle and to generate tests/golden fixtures; never shipped.
set -euo pipefail
REF=${DPGB_REFERENCE:-}
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
if [ -z "$REF" ] || [ ! -d "$REF/source/lib/src" ]; then
  echo "build_ref: DPGB_REFERENCE does not name a reference checkout; skipping" >&2
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

# The layout of the reference's backend-plugin interface (vtable slots of
# deepmd::DeepPotBackend, field offsets of deepmd::InputNlist), printed by
# tests/plugin/abi_probe.cc compiled against the reference's own headers,
# for tests/test_plugin_abi.py (the reference's common.h includes a header
# its build generates: an empty stand-in suffices here).
REPO_DIR="$(cd "$HERE/.." && pwd)"
mkdir -p "$OUT/probe"
printf '#pragma once\n' > "$OUT/probe/version.h"
g++ -std=c++17 -DPROBE_REFERENCE -I "$OUT/probe" -I "$REF/source/api_cc/include" -I "$REF/source/lib/include" \
  "$REPO_DIR/tests/plugin/abi_probe.cc" -o "$OUT/probe/abi_probe" && \
  "$OUT/probe/abi_probe" > "$OUT/abi_probe_reference.txt" && \
  echo "build_ref: wrote $OUT/abi_probe_reference.txt"
