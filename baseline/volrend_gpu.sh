#!/usr/bin/env bash
# The reference's own volume-rendering kernels (deps/volume-rendering-jax/lib/impl/{marching,
# integrating,packbits}.cu) and its spherical-harmonics kernel (deps/spherical-harmonics-encoding-
# jax/lib/impl/spherical_harmonics_encoding.cu), compiled unmodified for sm_103a with nvcc's default floating point
# (--fmad=true, as the reference's CMakeLists.txt builds them), into
# baseline/_ref/libvolrend_ref_gpu.so.  It is the GPU bar the new kernels are timed against and a
# GPU oracle for their parity tests; nothing in jaxngp_gb300/ loads it.
#
#   baseline/volrend_gpu.sh stage [REFERENCE_ROOT]   copy the sources out of the reference checkout
#                                                    into baseline/_ref/volrend_src (git-ignored; it
#                                                    travels to the GPU machine with the working tree)
#   baseline/volrend_gpu.sh build                    compile the staged sources (on any machine with
#                                                    nvcc; the library is built for the host it runs on)
#
# REFERENCE_ROOT defaults to $NGP_REFERENCE_ROOT, else /root/reference (the checkout's location in
# the build container).  `stage` exits 0 without doing anything when no checkout is found, and
# `build` exits 0 without doing anything when nothing was staged.
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
root="$(dirname "$here")"
src="$here/_ref/volrend_src"
out="$here/_ref"
cmd="${1:-build}"
case "$cmd" in
stage)
    ref="${2:-${NGP_REFERENCE_ROOT:-/root/reference}}"
    impl="$ref/deps/volume-rendering-jax/lib/impl"
    if [ ! -f "$impl/marching.cu" ]; then
        echo "volrend_gpu: no reference checkout at $ref; nothing staged" >&2
        exit 0
    fi
    mkdir -p "$src/impl" "$src/serde-helper"
    cp "$impl/marching.cu" "$impl/integrating.cu" "$impl/packbits.cu" "$impl/volrend.h" "$src/impl/"
    cp "$ref/deps/serde-helper/serde.h" "$src/serde-helper/"
    shsrc="$ref/deps/spherical-harmonics-encoding-jax/lib/impl"
    if [ -f "$shsrc/spherical_harmonics_encoding.cu" ]; then
        mkdir -p "$src/shjax"
        cp "$shsrc/spherical_harmonics_encoding.cu" "$shsrc/spherical_harmonics_encoding.h" "$src/shjax/"
    fi
    echo "staged $src"
    ;;
build)
    if [ ! -f "$src/impl/marching.cu" ]; then
        echo "volrend_gpu: nothing staged under $src; skipped" >&2
        exit 0
    fi
    nvcc="${NVCC:-$(command -v nvcc || echo /usr/local/cuda/bin/nvcc)}"
    flags=(-gencode arch=compute_103a,code=sm_103a -O3 -std=c++17 -Xcompiler -fPIC -w
           -I "$src" -I "$src/impl" -I "$root/oracle/ref_shim")
    mkdir -p "$out/obj"
    pids=()
    for k in marching integrating packbits; do
        "$nvcc" "${flags[@]}" -c "$src/impl/$k.cu" -o "$out/obj/$k.o" & pids+=($!)
    done
    shflag=()
    if [ -f "$src/shjax/spherical_harmonics_encoding.cu" ]; then
        "$nvcc" "${flags[@]}" -I "$src/shjax" -c "$src/shjax/spherical_harmonics_encoding.cu" -o "$out/obj/shjax.o" & pids+=($!)
        shflag=(-DNGP_REF_SHJAX -I "$src/shjax")
    fi
    "$nvcc" "${flags[@]}" "${shflag[@]}" -c "$here/volrend_gpu_exports.cu" -o "$out/obj/exports.o" & pids+=($!)
    for p in "${pids[@]}"; do wait "$p"; done
    "$nvcc" -gencode arch=compute_103a,code=sm_103a -shared -o "$out/libvolrend_ref_gpu.so.tmp" "$out"/obj/*.o
    mv "$out/libvolrend_ref_gpu.so.tmp" "$out/libvolrend_ref_gpu.so"
    echo "built $out/libvolrend_ref_gpu.so"
    ;;
*)
    echo "usage: $0 stage [REFERENCE_ROOT] | build" >&2
    exit 2
    ;;
esac
