#!/usr/bin/env bash
# Compile the reference's own volume-rendering kernels for the CPU, as a correctness oracle.
# TEST INFRASTRUCTURE ONLY.
#
# Each of deps/volume-rendering-jax/lib/impl/{marching,integrating,packbits}.cu is read where it
# lies under the reference checkout, its `<<<grid, block, smem, stream>>>` launch configurations
# are stripped on the fly (the launchers are never called), and it is compiled by g++ together
# with oracle/ref_shim/cuda_cpu_shim.h and the matching oracle/ref_driver_*.cpp, which runs every
# CUDA thread on the CPU.  Floating point is compiled with one rounding per operation
# (-ffp-contract=off), the reading of the CUDA source under nvcc --fmad=false.  Nothing of the
# reference is written to disk except the shared library oracle/_ref/libvolrend_ref_cpu.so.
#
# Usage: oracle/build_ref.sh [REFERENCE_ROOT]
# REFERENCE_ROOT defaults to $NGP_REFERENCE_ROOT, else /root/reference (the checkout's location in
# the build container); without a checkout the script builds nothing and exits 0.
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
ref="${1:-${NGP_REFERENCE_ROOT:-/root/reference}}"
impl="$ref/deps/volume-rendering-jax/lib/impl"
out="$here/_ref"
if [ ! -f "$impl/marching.cu" ]; then
    echo "build_ref: no reference checkout at $ref; nothing built" >&2
    exit 0
fi
mkdir -p "$out"
cuda_inc="${CUDA_HOME:-/usr/local/cuda}/include"
flags=(-std=c++20 -O2 -fPIC -ffp-contract=off -w -x c++
       -include "$here/ref_shim/cuda_cpu_shim.h" -I "$here/ref_shim" -I "$ref/deps"
       -I "$impl" -I "$cuda_inc")
objs=()
for k in marching integrating packbits; do
    { sed -E 's/<<<[^>]*>>>//g' "$impl/$k.cu"; cat "$here/ref_driver_$k.cpp"; } |
        g++ "${flags[@]}" -c -o "$out/$k.o" -
    objs+=("$out/$k.o")
done
g++ -std=c++20 -O2 -fPIC -I "$here/ref_shim" -I "$cuda_inc" -c -o "$out/runtime.o" \
    "$here/ref_shim/cuda_cpu_runtime.cpp"
g++ -shared -o "$out/libvolrend_ref_cpu.so" "${objs[@]}" "$out/runtime.o" -lpthread
rm -f "${objs[@]}" "$out/runtime.o"
echo "built $out/libvolrend_ref_cpu.so"
