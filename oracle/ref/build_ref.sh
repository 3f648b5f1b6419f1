#!/bin/sh
# Build the reference-side test tools from the read-only reference sources,
# where they lie (no copy is made), into oracle/_ref/:
#   libcy_ref.so   reference canvas + call-list replay (cyr_replay)
#   ref_recorder   the reference's own test/test.cpp compiled against the
#                  recording canvas (oracle/ref/recorder.hpp)
#   ref_tiger_recorder  the reference's tiger demo (demos/tiger/tiger.cpp)
#                  compiled against the same recording canvas
# Usage: oracle/ref/build_ref.sh REFERENCE_ROOT   (or CY_REFERENCE_ROOT in the environment)
set -e
REF=${1:-$CY_REFERENCE_ROOT}
if [ -z "$REF" ]; then
    echo "usage: $0 REFERENCE_ROOT (or set CY_REFERENCE_ROOT)" >&2
    exit 2
fi
HERE=$(cd "$(dirname "$0")" && pwd)
OUT=$HERE/../_ref
if [ ! -f "$REF/src/canvas_ity.hpp" ]; then
    echo "reference sources not found under $REF" >&2
    exit 2
fi
mkdir -p "$OUT/rec/src" "$OUT/rec/cwd"
FLAGS="-O3 -ffp-contract=off -fPIC"
g++ $FLAGS -shared -DCY_REFERENCE_HEADER="\"$REF/src/canvas_ity.hpp\"" \
    -o "$OUT/libcy_ref.so" "$HERE/ref_replay.cpp"
# test/test.cpp includes "../src/canvas_ity.hpp"; it is compiled from standard
# input inside $OUT/rec/cwd so that this include resolves to the recording
# header instead of the library header.
printf '#include "%s/recorder.hpp"\n' "$HERE" > "$OUT/rec/src/canvas_ity.hpp"
( cd "$OUT/rec/cwd" && g++ $FLAGS -Dmain=cy_test_main -x c++ -c -o "$OUT/rec/test.o" - < "$REF/test/test.cpp" )
g++ $FLAGS -DCY_REFERENCE_HEADER="\"$REF/src/canvas_ity.hpp\"" -c -o "$OUT/rec/recorder.o" "$HERE/recorder.cpp"
g++ -o "$OUT/ref_recorder" "$OUT/rec/test.o" "$OUT/rec/recorder.o"
# demos/tiger/tiger.cpp includes "../../src/canvas_ity.hpp": compiled from
# standard input two directories below $OUT/tiger, beside the recording header.
mkdir -p "$OUT/tiger/src" "$OUT/tiger/demo/cwd"
printf '#include "%s/recorder.hpp"\n' "$HERE" > "$OUT/tiger/src/canvas_ity.hpp"
( cd "$OUT/tiger/demo/cwd" && g++ $FLAGS -Dmain=cy_tiger_main -x c++ -c -o "$OUT/tiger/tiger.o" - < "$REF/demos/tiger/tiger.cpp" )
g++ $FLAGS -c -o "$OUT/tiger/tiger_main.o" "$HERE/tiger_main.cpp"
g++ -o "$OUT/ref_tiger_recorder" "$OUT/tiger/tiger.o" "$OUT/tiger/tiger_main.o" "$OUT/rec/recorder.o"
echo "built $OUT/libcy_ref.so $OUT/ref_recorder $OUT/ref_tiger_recorder"
