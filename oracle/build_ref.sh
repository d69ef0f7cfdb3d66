#!/bin/sh
# Builds the reference's own CPU code path into oracle/_ref/ (test infrastructure only).
#
#   ref_rec     the reference `2d_strip_reconstruction` tool, compiled straight from
#               src/2d/strip/reconstruction_cmd.cpp and its four helper translation
#               units with the reference's release flags (CMakeLists.txt:76,81) and
#               OpenMP; libpng is absent here, so ref_png_stub.cpp replaces
#               src/util/png_writer.cpp.  `-include cstdint` works around
#               src/util/bstream.h:7 using uint32_t without including <cstdint>.
#   ref_rec_strict  the same tool built with -ffp-contract=off.  The release
#               flags let GCC contract a*b+c into FMA in C++ mode on FMA-capable
#               hosts, so ref_rec's rounding depends on the host; the strict build
#               keeps the source's evaluation order and is what the CPU
#               restatement reproduces bit for bit.
#   ref_phantom the reference `2d_strip_phantom` event generator (same recipe).
#   ref_fp64    ref_fp64_harness.cpp: the reference Reconstruction template at double.
#   ref_analytic ref_analytic_harness.cpp: the reference AnalyticKernel and
#               Scanner::pixel_sensitivity at float and double (no FP contraction).
#   ref_hybrid  ref_hybrid_harness.cpp: the reference 3D hybrid Reconstruction
#               (src/3d/hybrid/reconstruction.h) on one thread, no FP contraction.
#   ref_convert the reference `3d_tool_convert` (src/3d/tool/convert_cmd.cpp with the
#               barrel and hybrid option files); MAX_DETECTORS=400 as the reference's
#               CMakeLists.txt:19 sets it.
#
# The reference's CMake project is not used (it does not configure with CMake 4).
# Sources are read in place from the reference checkout named by $JPET_REFERENCE
# (required; the build entry point sets it where the checkout exists); nothing is
# copied.  When the variable is unset or the sources are absent the script exits
# 0 and builds nothing.
set -e
REF=${JPET_REFERENCE:-}
if [ -z "$REF" ]; then
  echo "build_ref: JPET_REFERENCE is not set; skipping" >&2
  exit 0
fi
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
if [ ! -f "$REF/src/2d/strip/reconstruction_cmd.cpp" ]; then
  echo "build_ref: reference sources not found at $REF; skipping" >&2
  exit 0
fi
mkdir -p "$OUT"
CXX=${CXX:-g++}
ARCHFLAG=""
for f in -march=native -mcpu=native; do
  if echo 'int main(){return 0;}' | $CXX $f -x c++ - -o /dev/null 2>/dev/null; then
    ARCHFLAG=$f
    break
  fi
done
COMMON="-std=c++11 -O3 $ARCHFLAG -fopenmp -include cstdint -w \
  -I$REF/src -I$REF/lib/cmdline -I$REF/lib/json \
  -DUSE_FAST_TEXT_PARSER=1 -DUSE_SENSITIVITY=1 -DUSE_KERNEL=1 \
  -DUSE_STATISTICS=0 -DWARP_SIZE=32"
# the hybrid harness runs its event loop on one thread: no OpenMP
SERIAL="-std=c++11 -O3 $ARCHFLAG -include cstdint -w -I$REF/src -I$REF/lib/cmdline \
  -I$REF/lib/json -DUSE_FAST_TEXT_PARSER=1 -DMAX_DETECTORS=400 -DWARP_SIZE=32"
HELPERS="$REF/src/common/options.cpp $REF/src/util/cmdline_hooks.cpp \
  $REF/src/util/backtrace.cpp $REF/src/util/string.cpp $HERE/ref_png_stub.cpp"

$CXX $COMMON -o "$OUT/ref_rec" \
  "$REF/src/2d/strip/reconstruction_cmd.cpp" "$REF/src/2d/strip/options.cpp" \
  $HELPERS -ldl &
$CXX $COMMON -ffp-contract=off -o "$OUT/ref_rec_strict" \
  "$REF/src/2d/strip/reconstruction_cmd.cpp" "$REF/src/2d/strip/options.cpp" \
  $HELPERS -ldl &
$CXX $COMMON -o "$OUT/ref_phantom" \
  "$REF/src/2d/strip/phantom_cmd.cpp" "$REF/src/2d/strip/options.cpp" \
  $HELPERS -ldl &
$CXX $COMMON -ffp-contract=off -o "$OUT/ref_fp64" "$HERE/ref_fp64_harness.cpp" &
$CXX $COMMON -ffp-contract=off -o "$OUT/ref_analytic" "$HERE/ref_analytic_harness.cpp" &
$CXX $SERIAL -ffp-contract=off -o "$OUT/ref_hybrid" "$HERE/ref_hybrid_harness.cpp" &
$CXX $COMMON -DMAX_DETECTORS=400 -o "$OUT/ref_convert" \
  "$REF/src/3d/tool/convert_cmd.cpp" "$REF/src/3d/tool/options.cpp" \
  "$REF/src/2d/barrel/options.cpp" "$REF/src/3d/hybrid/options.cpp" $HELPERS -ldl &
wait
echo "build_ref: built $(ls "$OUT" | tr '\n' ' ')(flags: $ARCHFLAG)"
