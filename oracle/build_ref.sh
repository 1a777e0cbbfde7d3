#!/bin/sh
# Compiles the reference package's standalone-compilable sources, unchanged and
# where they lie, together with ref_probe.cpp into oracle/_ref/libmlipref.so.
# Test infrastructure only; needs the reference sources (REF_SRC) and g++.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
# REF_SRC: the reference package's src/USER-MLIP directory (required)
[ -n "$REF_SRC" ] || { echo "set REF_SRC to the reference's src/USER-MLIP directory" >&2; exit 2; }
OUT="$HERE/_ref"
[ -d "$REF_SRC" ] || { echo "reference sources not found: $REF_SRC" >&2; exit 2; }
mkdir -p "$OUT"
FLAGS="-std=c++17 -fPIC -I$REF_SRC"
SRCS="mlipkk_gtinv_data_reader mlipkk_irreps_type mlipkk_polynomial mlipkk_utils \
mlipkk_potential_parser mlipkk_spherical_harmonics mlipkk_cell"
pids=""
# the literal coupling table is large; -O0 keeps its compile time down
[ "$OUT/mlipkk_gtinv_data.o" -nt "$REF_SRC/mlipkk_gtinv_data.cpp" ] || \
  { g++ $FLAGS -O0 -c "$REF_SRC/mlipkk_gtinv_data.cpp" -o "$OUT/mlipkk_gtinv_data.o" & pids="$pids $!"; }
for s in $SRCS; do
  g++ $FLAGS -O2 -c "$REF_SRC/$s.cpp" -o "$OUT/$s.o" & pids="$pids $!"
done
g++ $FLAGS -O2 -c "$HERE/ref_probe.cpp" -o "$OUT/ref_probe.o" & pids="$pids $!"
for p in $pids; do wait $p; done
g++ -shared -o "$OUT/libmlipref.so" "$OUT"/*.o
echo "built $OUT/libmlipref.so"
