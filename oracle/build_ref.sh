#!/bin/sh
# Builds the reference's own sources (jy-yuan/sampling-graph-mining, read where they lie) into
# oracle/_ref/ for parity checks.  Test infrastructure: nothing in the product links these.
#
#   * src/*.cpp (except Random.cpp) + a replaying Random + single-rank MPI / one-node NUMA
#     shims  ->  one driver .so per application (oracle/ref/app_*.cpp include the app source);
#   * the same with the reference's own Random.cpp  ->  libzgtime_*.so, which time its
#     calculate() (oracle/ref/time_app.cpp; libzgtime_pattern.so: SamplerGenerator on a pattern);
#   * naive_implementation/*.cpp  ->  executables (with a zero-filling operator new[]);
#   * tests/Test{Pattern,Pattern2,Subgraph,Regression}.cpp  ->  executables.
#
# Skipped (exit 0) when the reference tree is absent, e.g. on a machine that only runs the
# committed golden fixtures.
set -e
REF=${ZG_REFERENCE_DIR:-/root/reference}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT=$HERE/_ref
if [ ! -d "$REF/src" ] || [ ! -d "$REF/applications" ]; then
  echo "build_ref: reference sources not found at $REF; skipping"
  exit 0
fi
mkdir -p "$OUT/obj" "$OUT/bin"
CXX=${CXX:-g++}
FLAGS="-O2 -std=c++14 -fopenmp -fPIC -fvisibility=hidden -w -include type_traits -include cstring"
INC="-I$HERE/ref/shim -I$REF/include -I$REF -I$HERE/ref"

for f in Bitmap Debug ErrorLatencyProfile Graph GraphFilters NetworkInterface Regression \
         SamplerGenerator SharedMemSys Time Type Utilities ZGraphInstance; do
  $CXX $FLAGS $INC -c "$REF/src/$f.cpp" -o "$OUT/obj/$f.o" &
done
$CXX $FLAGS $INC -c "$HERE/ref/replay_random.cpp" -o "$OUT/obj/replay_random.o" &
${CC:-gcc} -O2 -fopenmp -fPIC -fvisibility=hidden -c "$HERE/zg_oracle.c" -o "$OUT/obj/zg_oracle.o" &
wait

for app in triangle four_clique three_chain four_chain chain pred_triangle three_motif pattern; do
  $CXX $FLAGS $INC -shared -o "$OUT/libzgref_$app.so" "$HERE/ref/app_$app.cpp" "$OUT"/obj/*.o -lm &
done
wait

# timing drivers: the applications with the reference's own Random (mt19937) and OpenMP threads
mkdir -p "$OUT/obj_time"
$CXX $FLAGS $INC -c "$REF/src/Random.cpp" -o "$OUT/obj_time/Random.o"
TIME_OBJS=$(ls "$OUT"/obj/*.o | grep -v -e replay_random.o -e zg_oracle.o)
for pair in triangle:Triangle:TriangleCoutingInstance four_clique:FourClique:FourCliqueCountingInstance \
            three_chain:ThreeChain:ThreeChainCountingInstance four_chain:FourChain:FourChainCountingInstance; do
  app=${pair%%:*}; rest=${pair#*:}; file=${rest%%:*}; cls=${rest#*:}
  $CXX $FLAGS $INC -DZGREF_APP_FILE="\"applications/$file.cpp\"" -DZGREF_APP_CLASS=$cls -shared \
       -o "$OUT/libzgtime_$app.so" "$HERE/ref/time_app.cpp" $TIME_OBJS "$OUT/obj_time/Random.o" -lm &
done
$CXX $FLAGS $INC -DZGREF_PATTERN -shared -o "$OUT/libzgtime_pattern.so" "$HERE/ref/time_app.cpp" $TIME_OBJS \
     "$OUT/obj_time/Random.o" -lm &
wait

# naive exact counters (naive_implementation/Makefile builds them with plain g++)
mkdir -p "$OUT/naive_obj"
$CXX -O2 -c "$HERE/ref/zero_new.cpp" -o "$OUT/naive_obj/zero_new.o"
for c in TriangleCounting ThreeChain FourChain FiveChain FiveStar FourClique \
         WeightedTriangleCounting AtLeastOneWeightedTriangleCounting FiveHouse; do
  $CXX -O2 -fopenmp -w -include cstring -I"$HERE/ref/shim" "$REF/naive_implementation/$c.cpp" "$OUT/naive_obj/zero_new.o" \
       -o "$OUT/bin/naive_$c" &
done
wait

# the reference's own test programs (known answers for Pattern, SubGraph, regression)
for t in TestPattern TestPattern2 TestSubgraph TestRegression; do
  $CXX $FLAGS $INC "$REF/tests/$t.cpp" "$OUT"/obj/*.o -lm -o "$OUT/bin/$t" &
done
wait
missing=0
for f in "$OUT"/libzgref_triangle.so "$OUT"/libzgref_pattern.so "$OUT"/bin/naive_FiveHouse "$OUT"/bin/TestRegression; do
  [ -f "$f" ] || { echo "build_ref: missing $f"; missing=1; }
done
[ $missing -eq 0 ] || exit 1
echo "build_ref: built $OUT"
