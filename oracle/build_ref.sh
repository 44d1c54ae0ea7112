#!/usr/bin/env bash
# TEST INFRASTRUCTURE: builds the reference's own CPU tracer from its sources
# where they lie (read-only) into oracle/_ref/.  Nothing is copied from the
# reference tree.  Variants:
#   libemref_strict.so  -O3 -msse2 -fopenmp, IEEE arithmetic (no fast-math)
#   libemref_fast.so    the reference's release flags (CMakeLists.txt:24)
#   libemref_generic.so the scalar templates (no __SSE__)
#   libemref_inputs.so  the input generators of "Electromag utils.h"
# The reference's x86 path uses SSE intrinsics; on other architectures it
# falls back to the generic template (CPU_Implement.cpp:104-191) and the
# -msse2/-mfpmath flags do not exist, so they are only passed on x86.
set -euo pipefail
REF="${EM_REFERENCE_DIR:-/root/reference}"
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
SRC="$REF/ElectroMag/src/CPU_Implement.cpp"
if [ ! -f "$SRC" ]; then
    echo "build_ref.sh: reference sources not found at $REF" >&2
    exit 2
fi
mkdir -p "$OUT"
ARCHFLAGS=""
case "$(uname -m)" in
    x86_64|i?86) ARCHFLAGS="-msse2 -mfpmath=sse" ;;
esac
COMMON="-std=c++11 -O3 -DNDEBUG -fopenmp -fPIC -shared -ffp-contract=off \
  -D_GLIBCXX_USE_NANOSLEEP -I$REF/include -I$REF/ElectroMag/src"
g++ $COMMON $ARCHFLAGS "$SRC" "$HERE/ref_shim.cpp" -o "$OUT/libemref_strict.so"
g++ $COMMON $ARCHFLAGS -ffast-math -fno-math-errno -ffinite-math-only \
    "$SRC" "$HERE/ref_shim.cpp" -o "$OUT/libemref_fast.so"
# The generic scalar templates (CPU_Implement.cpp:38-191) that a build
# without __SSE__ runs (e.g. aarch64): undefining the macro selects them on
# x86 too, with the same IEEE scalar arithmetic.
g++ $COMMON $ARCHFLAGS -U__SSE__ "$SRC" "$HERE/ref_shim.cpp" \
    -o "$OUT/libemref_generic.so"
# The reference's input generators ("Electromag utils.h":29-111), header
# templates, with the C library's rand().
g++ $COMMON $ARCHFLAGS "$HERE/ref_inputs_shim.cpp" -o "$OUT/libemref_inputs.so"
echo "built $OUT/libemref_{strict,fast,generic,inputs}.so ($(uname -m))"
