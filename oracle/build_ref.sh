#!/usr/bin/env bash
# Builds the reference's own CPU path (ShugangZhang/LQT1) from its sources
# where they lie, into oracle/_ref/ (git-ignored).  TEST INFRASTRUCTURE ONLY.
#
# Nothing is copied: scenario variants are produced by streaming the
# reference's files through `sed` into the compiler.  Every patch is listed
# here and is limited to the scenario macros, the LQT1 factor, the stimulus
# duration, and (for the update() harness only) `private:` -> `public:` so that
# the harness can read and set the 40 states.
#
#   model_single_cell, model_oned          unmodified drivers, Makefile:20-35 flags
#   model_oned_cfg1                        OneD.cc + TPORd.cc with CON->LQT1, ISO1
#                                          off, GKs x0.5 (TPORd.cc:706) and a 2 ms
#                                          stimulus (OneD.cc:80)
# (TPORd.cc has CRLF line ends, hence the optional \r in the patterns.)
#   libtpord_ref_{default,baseline,lqt1,lqt1half,suprep}.so
#                                          TPORd.cc + oracle/ref_harness.inc
#   libgrid_ref_{2d,3d}.so                 line ranges of new_11.cu / GPU3D.cu
#                                          (constants with a smaller grid,
#                                          get_u_v, calc_du, the mirror-map
#                                          loop) + oracle/ref_grid_harness.inc
#
# Usage: oracle/build_ref.sh REFERENCE_DIR   (or LQT_REFERENCE=REFERENCE_DIR)
set -euo pipefail
REF=${1:-${LQT_REFERENCE:-}}
[ -n "$REF" ] || { echo "usage: $0 REFERENCE_DIR (a checkout of ShugangZhang/LQT1)" >&2; exit 2; }
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
[ -f "$REF/SingleCell/TPORd.cc" ] || { echo "reference not found at $REF" >&2; exit 2; }
mkdir -p "$OUT"
CXX=${CXX:-g++}
TPORD="$REF/SingleCell/TPORd.cc"

# 1. unmodified drivers (Makefile:30-35 recipes; target SingleCell is shadowed
#    by the SingleCell/ directory in the reference's make, so it is built here).
$CXX -w -O3 -o "$OUT/model_single_cell" "$REF/SingleCell/Cell.cc" "$TPORD" "$REF/SingleCell.cc" &
$CXX -w -O3 -fopenmp -o "$OUT/model_oned" "$REF/SingleCell/Cell.cc" "$TPORD" "$REF/OneD.cc" &

# 2. scenario variant of the 1D driver for the 1D strand workload.
SCEN_LQT1HALF=(-e 's|^#define CON\r\?$|#define LQT1|' -e 's|^#define ISO1\r\?$|// ISO1 off|' \
               -e 's|GKs = 0.05\*GKs;|GKs = 0.5*GKs;|')
{ sed "${SCEN_LQT1HALF[@]}" "$TPORD"
  sed -e 's|^#include "SingleCell/TPORd.cc"|// TPORd streamed above|' \
      -e 's|double stimDuration = 1.0;|double stimDuration = 2.0;|' "$REF/OneD.cc"; } |
  $CXX -w -O3 -fopenmp -x c++ -I"$REF/SingleCell" -o "$OUT/model_oned_cfg1" - &

# 3. update() harness, one library per scenario.
harness() {
  local name=$1; shift
  { sed -e 's|^private:\r\?$|public:|' "$@" "$TPORD"; cat "$HERE/ref_harness.inc"; } |
    $CXX -w -O3 -fPIC -shared -fopenmp -x c++ -I"$REF/SingleCell" -o "$OUT/libtpord_ref_$name.so" -
}
harness default -e 's|^//__none__||' &
harness baseline -e 's|^#define CON\r\?$|#define BASELINE|' -e 's|^#define ISO1\r\?$|// ISO1 off|' &
harness lqt1 -e 's|^#define CON\r\?$|#define LQT1|' -e 's|^#define ISO1\r\?$|// ISO1 off|' &
harness lqt1half "${SCEN_LQT1HALF[@]}" &
harness suprep -e 's|^// #define SUPREP\r\?$|#define SUPREP|' &

# 4. the reference's own 2D/3D stencil and mirror-map lines (new_11.cu,
#    GPU3D.cu) on small grids: constants with X/Y/Z patched, get_u_v, calc_du,
#    and the map loop of main() streamed into oracle/ref_grid_harness.inc.
gridref() {
  local name=$1 src=$2 dim=$3 consts=$4 getuv=$5 calcdu=$6 maploop=$7 filld=$8; shift 8
  local tmp; tmp=$(mktemp -d)
  sed -n "${maploop}p" "$REF/$src" > "$tmp/map_loop.inc"
  if [ -n "$filld" ]; then sed -n "${filld}p" "$REF/$src" > "$tmp/fill_d.inc"; fi
  { printf '#include <cmath>\n#include <iostream>\nusing namespace std;\n'
    printf '#define __global__\n#define __device__\nstruct LqtDim3 { int x, y, z; };\n'
    printf 'static LqtDim3 blockIdx, blockDim, threadIdx;\n#define LQT_REF_DIM %s\n' "$dim"
    printf '#define LQT_REF_MAP_LOOP "%s/map_loop.inc"\n#define LQT_REF_FILL_D "%s/fill_d.inc"\n' "$tmp" "$tmp"
    sed -n "${consts}p" "$REF/$src" | sed "$@"
    sed -n "${getuv}p" "$REF/$src"
    sed -n "${calcdu}p" "$REF/$src"
    cat "$HERE/ref_grid_harness.inc"; } |
    $CXX -w -O2 -ffp-contract=off -fPIC -shared -x c++ -o "$OUT/libgrid_ref_$name.so" -
  rm -rf "$tmp"
}
gridref 2d new_11.cu 2 29,63 234,284 352,417 1535,1689 1496,1499 \
  -e 's|^const int X = 690;|const int X = 44;|' -e 's|^const int Y = 489;|const int Y = 38;|' &
gridref 3d GPU3D.cu 3 28,42 258,308 370,385 1487,1680 "" \
  -e 's|^const int X = 690;|const int X = 24;|' -e 's|^const int Y = 489;|const int Y = 22;|' \
  -e 's|^const int Z = 537;|const int Z = 28;|' &
wait
echo "reference built into $OUT"
