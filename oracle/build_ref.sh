#!/usr/bin/env bash
# Builds the unmodified reference engine (rlguy/Blender-FLIP-Fluids, src/engine) into
# oracle/_ref/libffengine.so and the golden-vector harness oracle/_ref/ref_harness.
#
# Test infrastructure only: the product never links or loads anything under oracle/_ref.
# The reference sources are compiled where they lie (read-only); only build outputs are
# written, and only into oracle/_ref/.  Flags follow the reference's Linux build
# (CMakeLists.txt:137) minus the x86-only glibc symver header, with -ffp-contract=off so
# that a non-x86 host computes the same floats as the reference's x86-64 build.
#
# Usage: oracle/build_ref.sh REFERENCE_ROOT   (or set FFGPU_REFERENCE_ROOT)
set -euo pipefail
REF="${1:-${FFGPU_REFERENCE_ROOT:-}}"
if [ -z "$REF" ]; then
    echo "usage: $0 REFERENCE_ROOT (the rlguy/Blender-FLIP-Fluids checkout)" >&2
    exit 2
fi
ENG="$REF/src/engine"
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
OBJ="$OUT/obj"
if [ ! -d "$ENG" ]; then
    echo "reference engine sources not found at $ENG" >&2
    exit 2
fi
mkdir -p "$OBJ"
CXXFLAGS="-std=c++17 -O3 -fopenmp -fPIC -pthread -ffp-contract=off -DWITH_MIXBOX=0 -D_GLIBCXX_USE_NANOSLEEP -w -I$ENG -I$ENG/c_bindings"

# versionutils.cpp.in -> configured copy (6 substitutions, versionutils.cpp.in:27-32)
sed -e 's/@FFENGINE_VERSION_MAJOR@/1/' -e 's/@FFENGINE_VERSION_MINOR@/8/' \
    -e 's/@FFENGINE_VERSION_REVISION@/5/' -e 's/@FFENGINE_VERSION_LABEL@/ref/' \
    -e 's/@FFENGINE_VERSION_SUPPORT_LICENSE_TYPE@/none/' \
    -e 's/@FFENGINE_VERSION_SUPPORT_LICENSE_ID@/none/' \
    "$ENG/versionutils.cpp.in" > "$OBJ/versionutils_configured.cpp"

SRCS=()
for f in "$ENG"/*.cpp "$ENG"/c_bindings/*.cpp "$ENG"/mixbox/mixbox_stub.cpp; do
    case "$(basename "$f")" in main.cpp) continue ;; esac
    SRCS+=("$f")
done
SRCS+=("$OBJ/versionutils_configured.cpp")

pids=()
objs=()
for f in "${SRCS[@]}"; do
    o="$OBJ/$(echo "$f" | sed 's#[/.]#_#g').o"
    objs+=("$o")
    if [ ! -f "$o" ] || [ "$f" -nt "$o" ]; then
        g++ $CXXFLAGS -c "$f" -o "$o" &
        pids+=($!)
        if [ "${#pids[@]}" -ge "$(nproc)" ]; then wait "${pids[0]}"; pids=("${pids[@]:1}"); fi
    fi
done
for p in "${pids[@]}"; do wait "$p"; done
g++ -shared -fopenmp -pthread -o "$OUT/libffengine.so" "${objs[@]}"

g++ $CXXFLAGS -I"$ENG" "$HERE/ref_harness.cpp" -o "$OUT/ref_harness" \
    -L"$OUT" -lffengine -Wl,-rpath,"$OUT"
echo "built $OUT/libffengine.so and $OUT/ref_harness"
