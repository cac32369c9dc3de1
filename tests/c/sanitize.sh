#!/bin/bash
# AddressSanitizer / UndefinedBehaviorSanitizer run of the host layer (needs a GPU):
# an instrumented copy of libgsks.so in tests/c/_build/asan, and the C and C++ callers
# of tests/c linked to it and run in both precisions.  Run from the repository root:
#     bash tests/c/sanitize.sh
set -e
D=tests/c/_build/asan; mkdir -p $D/obj
ARCH="-gencode arch=compute_103a,code=sm_103a"
F="-O1 -g -std=c++17 --expt-relaxed-constexpr -Iinclude -Iks_gb300/csrc -Xcompiler -fPIC,-fopenmp,-fsanitize=address,-fsanitize=undefined,-fno-omit-frame-pointer"
pids=()
for f in ks_gb300/csrc/*.cu ks_gb300/csrc/*.cpp; do
  b=$(basename $f)
  if [[ $f == *.cpp ]]; then nvcc -x cu $ARCH $F -c $f -o $D/obj/$b.o & else nvcc $ARCH $F -c $f -o $D/obj/$b.o & fi
  pids+=($!)
done
for p in ${pids[@]}; do wait $p; done
nvcc $ARCH -shared -o $D/libgsks.so $D/obj/*.o -Xcompiler -fopenmp,-fsanitize=address,-fsanitize=undefined -lgomp -ldl
S="-fsanitize=address,undefined -fno-omit-frame-pointer -g"
gcc $S -Iinclude tests/c/link_dgsks.c -o $D/link_dgsks -L$D -lgsks -Wl,-rpath,$PWD/$D -lm
g++ $S -Iinclude tests/c/link_list.cpp -o $D/link_list -L$D -lgsks -Wl,-rpath,$PWD/$D
g++ $S -Iinclude tests/c/list_signatures.cpp -o $D/list_signatures -L$D -lgsks -Wl,-rpath,$PWD/$D
python - <<'PY'
import numpy as np
rng = np.random.default_rng(1); N, k, nt = 1500, 7, 6
sa = rng.integers(0, 300, nt); sb = rng.integers(0, 200, nt)
a = np.concatenate([rng.permutation(N)[:s] for s in sa]).astype(np.int32)
u = np.concatenate([rng.permutation(N)[:s] for s in sa]).astype(np.int32)
b = np.concatenate([rng.permutation(N)[:s] for s in sb]).astype(np.int32)
wi = rng.integers(0, N, b.size).astype(np.int32)
with open("tests/c/_build/asan/in.bin", "wb") as f:
    np.array([N, N, k, nt, N, N], np.int32).tofile(f); np.array([2, 0, 0, 1], np.float64).tofile(f)
    for x in (rng.random((N, k)), rng.random((N, k)), rng.standard_normal(N), rng.standard_normal(N)): x.tofile(f)
    for x in (np.concatenate([[0], np.cumsum(sa)]), a, u, np.concatenate([[0], np.cumsum(sb)]), b, wi): x.astype(np.int32).tofile(f)
PY
export ASAN_OPTIONS=protect_shadow_gap=0:detect_leaks=0:halt_on_error=1
export UBSAN_OPTIONS=print_stacktrace=1:halt_on_error=1
for P in "fp64" "split"; do
  export GSKS_PRECISION=$P
  $D/link_dgsks > $D/o1_$P.txt
  $D/link_list > $D/o2_$P.txt
  $D/list_signatures $D/in.bin $D/o3_$P.bin
  echo "asan/ubsan clean: $P"
done
