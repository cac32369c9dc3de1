#!/usr/bin/env bash
# Builds the reference GSKS library (ChenhanYu/ks) from its own sources, in
# place, into oracle/_ref/.  Test infrastructure only: the result is the
# checker the parity tests and the golden-vector generator compare against.
#
# Recipe (x86_64 only; the reference's micro-kernels are AVX intrinsics):
#   * micro_kernel/x86_64/sandybridge/*  -- the kernel list of the reference
#     makefile (makefile:15-34), gcc -O3 -mavx2 -mfma.
#   * frame/dgsks.c                      -- compiled WITHOUT -fopenmp and with
#     omp_get_thread_num() defined to 0: its two `omp parallel for` loops
#     (dgsks.c:486,619) are not in OpenMP canonical form, and a threaded
#     dgsks called from omp_dgsks_list indexes packu by the outer thread id.
#   * frame/dgsks_ref.c, frame/ks_util.c, frame/omp_dgsks_list.cpp -- -fopenmp.
#   * linked with g++ -shared (omp_dgsks_list.cpp needs libstdc++).
# USE_BLAS and USE_VML stay off (no CPU BLAS / MKL in the image), so
# dgsks_ref runs its naive GEMM loops with glibc exp/pow/tanh.
set -euo pipefail
REF=${GSKS_REFERENCE:-/root/reference}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
if [ ! -f "$REF/include/ks.h" ]; then
  echo "build_ref.sh: reference sources not found at $REF" >&2; exit 2
fi
if [ "$(uname -m)" != "x86_64" ]; then
  echo "build_ref.sh: the reference micro-kernels need x86_64 (AVX)" >&2; exit 3
fi
mkdir -p "$OUT/obj"
MK="$REF/micro_kernel/x86_64/sandybridge"
INC="-I$REF/include -I$MK"
CF="-O3 -fPIC -mavx2 -mfma -w"
objs=()
for f in ks_gaussian_int_d8x4 ks_gaussian_svml_d8x4 ks_variable_bandwidth_gaussian_int_d8x4 \
         ks_polynomial_int_d8x4 ks_laplace3d_int_d8x4 ks_tanh_int_d8x4 ks_quartic_int_d8x4 \
         ks_epanechnikov_int_d8x4 ks_multiquadratic_int_d8x4 ks_rank_k_int_d8x4 ks_rank_k_asm_d8x4; do
  gcc $CF $INC -c "$MK/$f.c" -o "$OUT/obj/$f.o" &
  objs+=("$OUT/obj/$f.o")
done
gcc $CF $INC "-Domp_get_thread_num()=0" -c "$REF/frame/dgsks.c" -o "$OUT/obj/dgsks.o" &
gcc $CF -fopenmp $INC -c "$REF/frame/dgsks_ref.c" -o "$OUT/obj/dgsks_ref.o" &
gcc $CF -fopenmp $INC -c "$REF/frame/ks_util.c" -o "$OUT/obj/ks_util.o" &
g++ $CF -fopenmp $INC -c "$REF/frame/omp_dgsks_list.cpp" -o "$OUT/obj/omp_dgsks_list.o" &
wait
objs+=("$OUT/obj/dgsks.o" "$OUT/obj/dgsks_ref.o" "$OUT/obj/ks_util.o" "$OUT/obj/omp_dgsks_list.o")
g++ -shared -fopenmp -o "$OUT/libgsks_ref.so" "${objs[@]}" -lm
echo "built $OUT/libgsks_ref.so"
# Flat C shim over the reference's C++ list driver (our own file, linked
# against the reference library built above).
g++ -O2 -fPIC -shared -w -I"$REF/include" "$HERE/ref_list_shim.cpp" \
    -o "$OUT/libref_list_shim.so" -L"$OUT" -lgsks_ref -Wl,-rpath,'$ORIGIN'
echo "built $OUT/libref_list_shim.so"
