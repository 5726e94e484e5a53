#!/usr/bin/env bash
# build_ref_gpu.sh - compile the reference's CUDA backend (every .cu under
# Spike/Backend) for this GPU together with its front end (Spike/Models,
# Neurons, Synapses, Plasticity, ActivityMonitor, Helpers, Backend/Context and
# the Dummy backend), and link them with oracle/ref_gpu_run.cpp into
# oracle/_ref/gpu/ref_gpu_run.
#
# TEST INFRASTRUCTURE ONLY.  The reference's CMake build is not used (it needs
# FindCUDA and targets sm_37).  Objects are built from the source files where
# they lie; nothing of the reference is copied into the repository, and the
# outputs go to oracle/_ref/gpu/ (git-ignored).  The objects are linked as the
# reference's backend registration needs: front-end objects first (they
# define the factory maps), then the Dummy and CUDA backends as whole
# archives, then the device-link object and the CUDA runtime.
#
# Usage: oracle/build_ref_gpu.sh REFERENCE_ROOT [ARCH]   (ARCH default sm_103a)
#
# REF_STRICT_FP=1 compiles every float expression as written: no fused
# multiply-add on the device (-fmad=false) or the host (-ffp-contract=off),
# the convention of the oracle and of this library.  The outputs then go to
# oracle/_ref/gpu_strict/ instead.
set -euo pipefail
REF="${1:?usage: build_ref_gpu.sh REFERENCE_ROOT [ARCH]}"
ARCH="${2:-sm_103a}"
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref/gpu"
STRICT="${REF_STRICT_FP:-0}"
[ "$STRICT" = 1 ] && OUT="$HERE/_ref/gpu_strict"
if [ ! -d "$REF/Spike/Backend/CUDA" ]; then
  echo "build_ref_gpu: no reference CUDA backend under $REF" >&2
  exit 1
fi
NVCC="${NVCC:-nvcc}"
CUDA_HOME="$(cd "$(dirname "$(command -v "$NVCC")")/.." && pwd)"
CXX="${CXX:-g++}"
mkdir -p "$OUT/obj"
DEF='-DSPIKE_DEFAULT_BACKEND="CUDA"'
CXXFLAGS=(-std=c++11 -O2 -w -fPIC -I"$REF" -I"$CUDA_HOME/include" -DNDEBUG "$DEF")
NVFLAGS=(-std=c++11 -O2 -w -gencode "arch=compute_${ARCH#sm_},code=$ARCH" -I"$REF" -Xcompiler -fPIC "$DEF")
if [ "$STRICT" = 1 ]; then
  CXXFLAGS+=(-ffp-contract=off)
  NVFLAGS+=(-fmad=false -Xcompiler -ffp-contract=off)
fi

front=(); dummy=(); cuda=()
while IFS= read -r f; do front+=("$f"); done < <(
  { echo "$REF/Spike/Backend/Context.cpp";
    find "$REF/Spike/Helpers" "$REF/Spike/Models" "$REF/Spike/Neurons" "$REF/Spike/Plasticity" \
         "$REF/Spike/ActivityMonitor" "$REF/Spike/Synapses" -name '*.cpp'; } | sort)
while IFS= read -r f; do dummy+=("$f"); done < <(find "$REF/Spike/Backend/Dummy" -name '*.cpp' | sort)
while IFS= read -r f; do cuda+=("$f"); done < <(find "$REF/Spike/Backend" -name '*.cu' | sort)

JOBS="${JOBS:-$(nproc)}"
pids=()
wait_some() {  # keep at most JOBS compilers running
  while [ "$(jobs -rp | wc -l)" -ge "$JOBS" ]; do sleep 0.2; done
}
i=0; of=(); od=(); oc=()
for f in "${front[@]}"; do o="$OUT/obj/f$i.o"; of+=("$o"); i=$((i + 1)); wait_some
  "$CXX" "${CXXFLAGS[@]}" -c "$f" -o "$o" & pids+=($!); done
for f in "${dummy[@]}"; do o="$OUT/obj/d$i.o"; od+=("$o"); i=$((i + 1)); wait_some
  "$CXX" "${CXXFLAGS[@]}" -c "$f" -o "$o" & pids+=($!); done
for f in "${cuda[@]}"; do o="$OUT/obj/c$i.o"; oc+=("$o"); i=$((i + 1)); wait_some
  "$NVCC" "${NVFLAGS[@]}" -dc "$f" -o "$o" & pids+=($!); done
wait_some
"$CXX" "${CXXFLAGS[@]}" -c "$HERE/ref_gpu_run.cpp" -o "$OUT/obj/run.o" & pids+=($!)
for p in "${pids[@]}"; do wait "$p"; done

"$NVCC" -gencode "arch=compute_${ARCH#sm_},code=$ARCH" -Xcompiler -fPIC -dlink "${oc[@]}" -o "$OUT/obj/dlink.o" -lcudadevrt
"$CXX" -o "$OUT/ref_gpu_run" "$OUT/obj/run.o" "${of[@]}" \
  -Wl,--whole-archive "${od[@]}" "${oc[@]}" -Wl,--no-whole-archive "$OUT/obj/dlink.o" \
  -L"$CUDA_HOME/lib64" -L"$CUDA_HOME/lib" -lcudadevrt -lcudart -lpthread -ldl -lrt
echo "build_ref_gpu: built $OUT/ref_gpu_run"
