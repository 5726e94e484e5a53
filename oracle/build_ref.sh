#!/usr/bin/env bash
# build_ref.sh - compile the reference's own front end (Spike/Models, Neurons,
# Synapses, Plasticity, ActivityMonitor, Helpers, Backend/Context) and its
# Dummy backend straight from the reference sources with g++, and link them
# with oracle/ref_dump.cpp (and the case builders it includes,
# oracle/ref_cases.inc) into oracle/_ref/ref_dump.
#
# TEST INFRASTRUCTURE ONLY.  The reference's CMake build is not used (it
# requires FindCUDA); no reference source is copied: objects are built from
# the files where they lie.  Outputs go to oracle/_ref/ (git-ignored).
#
# Usage: oracle/build_ref.sh [REFERENCE_ROOT]
# The root is the argument, else $SPIKE_REFERENCE_ROOT, else the reference's
# checkout on the development machine (/root/reference).  Without the sources
# there the recipe builds nothing and exits 0 (machines without the reference,
# such as the GPU hosts, use the committed fixtures only).
set -euo pipefail
REF="${1:-${SPIKE_REFERENCE_ROOT:-/root/reference}}"
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
if [ ! -d "$REF/Spike" ]; then
  echo "build_ref: no reference sources at $REF; nothing built" >&2
  exit 0
fi
mkdir -p "$OUT/obj"
CXX="${CXX:-g++}"
FLAGS=(-std=c++11 -O1 -w -I"$REF" -DNDEBUG "-DSPIKE_DEFAULT_BACKEND=\"Dummy\"")

front=()
while IFS= read -r f; do front+=("$f"); done < <(
  { echo "$REF/Spike/Backend/Context.cpp";
    find "$REF/Spike/Helpers" "$REF/Spike/Models" "$REF/Spike/Neurons" "$REF/Spike/Plasticity" \
         "$REF/Spike/ActivityMonitor" "$REF/Spike/Synapses" -name '*.cpp'; } | sort)
dummy=()
while IFS= read -r f; do dummy+=("$f"); done < <(find "$REF/Spike/Backend/Dummy" -name '*.cpp' | sort)

objs_front=()
objs_dummy=()
compile() {  # src obj
  "$CXX" "${FLAGS[@]}" -c "$1" -o "$2"
}
pids=()
i=0
for f in "${front[@]}"; do
  o="$OUT/obj/front_$i.o"; objs_front+=("$o"); i=$((i + 1))
  compile "$f" "$o" & pids+=($!)
done
for f in "${dummy[@]}"; do
  o="$OUT/obj/dummy_$i.o"; objs_dummy+=("$o"); i=$((i + 1))
  compile "$f" "$o" & pids+=($!)
done
"$CXX" "${FLAGS[@]}" -c "$HERE/ref_dump.cpp" -o "$OUT/obj/ref_dump.o" & pids+=($!)
for p in "${pids[@]}"; do wait "$p"; done

# Front-end objects first, then the Dummy backend: the backend registrars
# write into factory maps defined in front-end translation units.
"$CXX" -o "$OUT/ref_dump" "$OUT/obj/ref_dump.o" "${objs_front[@]}" \
  -Wl,--whole-archive "${objs_dummy[@]}" -Wl,--no-whole-archive
echo "build_ref: built $OUT/ref_dump"
