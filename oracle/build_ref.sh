#!/usr/bin/env bash
# Compiles the reference's OWN C++ sources, unchanged, where they lie under
# /root/reference, against the stand-in headers in oracle/shim/ (FFTW and
# Boost are not installed here), into the reference CLI (golay_ref) and the
# window driver of oracle/ref_window_driver.cpp (golay_ref_window).  Output
# goes only to oracle/_ref/.
#
# Test infrastructure: the resulting binary cross-checks the oracle
# restatement and generates golden files.  It is never shipped and never run
# by the product path.  It only exists where /root/reference exists.
set -euo pipefail
REF=${GP_REFERENCE_DIR:-/root/reference}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
if [ ! -d "$REF/src" ]; then
    echo "build_ref: no reference sources at $REF; skipping" >&2
    exit 0
fi
mkdir -p "$OUT/obj"
SRCS=(
    src/main.cpp
    src/utils/array.cpp src/utils/binary.cpp src/utils/coprimes.cpp src/utils/decomps.cpp
    src/utils/equivalence.cpp src/utils/fourier.cpp src/utils/golay.cpp src/utils/io.cpp
    src/utils/lyndon.cpp src/utils/orderly_equivalence.cpp
    src/core/generate/generate_hybrid.cpp src/core/filter/filter.cpp src/core/match/match_pairs.cpp
    src/core/sort/sort.cpp src/core/uncompression/uncompression.cpp
)
INC=(-I"$HERE/shim" -I"$REF/src/utils" -I"$REF/src/core/generate" -I"$REF/src/core/filter"
     -I"$REF/src/core/match" -I"$REF/src/core/sort" -I"$REF/src/core/uncompression"
     -I"$REF/src/core/uncompression/gpu" -I"$REF/third_party")
OBJS=()
pids=()
for s in "${SRCS[@]}"; do
    o="$OUT/obj/$(echo "$s" | tr '/' '_' | sed 's/\.cpp$/.o/')"
    OBJS+=("$o")
    if [ ! -f "$o" ] || [ "$REF/$s" -nt "$o" ] || [ "$HERE/build_ref.sh" -nt "$o" ]; then
        g++ -std=c++20 -O2 -w "${INC[@]}" -c "$REF/$s" -o "$o" &
        pids+=($!)
    fi
done
for p in "${pids[@]}"; do wait "$p"; done
g++ -O2 -o "$OUT/golay_ref" "${OBJS[@]}" -lm
# the window driver (oracle/ref_window_driver.cpp) over the same objects, minus main
DRV="$OUT/obj/ref_window_driver.o"
g++ -std=c++20 -O2 -w "${INC[@]}" -c "$HERE/ref_window_driver.cpp" -o "$DRV"
g++ -O2 -o "$OUT/golay_ref_window" "$DRV" "${OBJS[@]:1}" -lm
echo "build_ref: built $OUT/golay_ref and $OUT/golay_ref_window"
