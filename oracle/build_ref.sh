#!/bin/sh
# Builds oracle/_ref/libpars_ref.so: the reference's own hot-path sources,
# compiled unmodified from the reference checkout, against the stand-ins in
# oracle/ref_shim/include and the reference's vendored Eigen 3.3.7.
# Usage: oracle/build_ref.sh [reference-root]
# (default: $PARS_REFERENCE, else a `reference` directory beside the repository)
# Default x86-64 code generation (SSE2, no FMA) matches the reference build
# flags (pa/CMakeLists.txt:37-43).
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${1:-${PARS_REFERENCE:-$(dirname "$(dirname "$HERE")")/reference}}
OUT="$HERE/_ref"
[ -d "$REF/pa/source" ] || { echo "reference sources not found under $REF" >&2; exit 1; }
mkdir -p "$OUT"
FLAGS="-std=c++17 -O2 -fopenmp -DNDEBUG -fPIC -w -ffp-contract=off -I$HERE/ref_shim/include -I$REF/pa/include -I$REF/pa/include/external"
OBJS=""
for f in math/vector_field stages/particle_tracer stages/particle_advector stages/flow_map_generator \
         stages/ftle_map_generator stages/index_generator stages/color_generator stages/seed_generator stages/partitioner; do
  o="$OUT/$(basename $f).o"
  g++ $FLAGS -c "$REF/pa/source/$f.cpp" -o "$o" &
  OBJS="$OBJS $o"
done
g++ $FLAGS -c "$HERE/ref_driver.cpp" -o "$OUT/ref_driver.o" &
wait
g++ -shared -fopenmp -o "$OUT/libpars_ref.so" $OBJS "$OUT/ref_driver.o"
echo "built $OUT/libpars_ref.so"
