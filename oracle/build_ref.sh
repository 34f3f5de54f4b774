#!/usr/bin/env bash
# build_ref.sh -- compile the reference's host render path, in place, into
# oracle/_ref/ (test infrastructure only: the checker, never the product).
#
# Reads the reference sources where they lie ($SPLOTCH_REF_DIR, else the
# reference checkout named below -- the one place that names it) and writes
# only under oracle/_ref/.  `build_ref.sh --where` prints that location.
# Two libraries and one PTX module:
#   libsplotch_ref.so         default flags (on x86-64 __SSE2__ is defined, so
#                             render_new takes its V4sf absorption branch)
#   libsplotch_ref_scalar.so  the same with -U__SSE2__: the scalar branch that
#                             an AArch64 (Grace) host compiles
#   legacy_cuda_kernel.ptx    the legacy GPU kernels (cuda/cuda_kernel.cu), run by
#                             oracle/legacy_gpu.cc as the GPU floor
# Flags follow the reference's own plain build without -Ofast: -O2 -fopenmp,
# plus -ffp-contract=off so no fused multiply-add changes its rounding.
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF="${SPLOTCH_REF_DIR:-/root/reference}"
if [ "${1:-}" = "--where" ]; then echo "$REF"; exit 0; fi
OUT="$HERE/_ref"
if [ ! -f "$REF/splotch/splotch_host.cc" ]; then
  echo "reference sources not found at $REF; skipping oracle/_ref" >&2
  exit 0
fi
mkdir -p "$OUT"
SRCS=(splotch/splotch_host.cc splotch/splotchutils.cc splotch/new_renderer.cc
      kernel/transform.cxx cxxsupport/paramfile.cc cxxsupport/error_handling.cc
      cxxsupport/string_utils.cc cxxsupport/mpi_support.cc cxxsupport/walltimer.cc
      cxxsupport/announce.cc cxxsupport/ls_image.cc splotch/scenemaker.cc)
CXXFLAGS=(-O2 -std=c++11 -fopenmp -ffp-contract=off -fPIC -w
          -I"$REF" -I"$REF/cxxsupport" -I"$REF/c_utils")

build_variant() {  # $1 = output name, $2.. = extra flags
  local name="$1"; shift
  local obj="$OUT/obj_$name"
  mkdir -p "$obj"
  local pids=() objs=()
  for s in "${SRCS[@]}"; do
    local o="$obj/$(basename "$s").o"
    objs+=("$o")
    g++ "${CXXFLAGS[@]}" "$@" -c "$REF/$s" -o "$o" & pids+=($!)
  done
  gcc -O2 -fPIC -ffp-contract=off "$@" -I"$REF/c_utils" -c "$REF/c_utils/walltime_c.c" \
      -o "$obj/walltime_c.o" & pids+=($!)
  g++ "${CXXFLAGS[@]}" "$@" -c "$HERE/ref_harness.cc" -o "$obj/ref_harness.o" & pids+=($!)
  g++ "${CXXFLAGS[@]}" "$@" -c "$HERE/ref_stubs.cc" -o "$obj/ref_stubs.o" & pids+=($!)
  for p in "${pids[@]}"; do wait "$p"; done
  g++ -shared -fopenmp -Wl,--no-undefined -o "$OUT/$name.so" "${objs[@]}" \
      "$obj/walltime_c.o" "$obj/ref_harness.o" "$obj/ref_stubs.o"
}

build_variant libsplotch_ref
build_variant libsplotch_ref_scalar -U__SSE2__
# The reference's legacy GPU kernels (cuda/cuda_kernel.cu, whose header
# selects the full-atomics renderer and the classic kernel) as PTX for sm_103a:
# text that the GPU host's driver compiles when oracle/legacy_gpu.cc loads it.
# Flags of the reference's generic CUDA build (Makefile: -std=c++11, no fast
# math), without its relocatable-device-code split: the one file holds every
# kernel and constant it needs.
NVCC="${NVCC:-$(command -v nvcc || echo /usr/local/cuda/bin/nvcc)}"
"$NVCC" -ptx -arch=compute_103a -std=c++11 -I"$REF" -I"$REF/cxxsupport" -I"$REF/c_utils" \
    "$REF/cuda/cuda_kernel.cu" -o "$OUT/legacy_cuda_kernel.ptx"
echo "built $OUT/libsplotch_ref.so $OUT/libsplotch_ref_scalar.so $OUT/legacy_cuda_kernel.ptx"
