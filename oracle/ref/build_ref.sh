#!/usr/bin/env bash
# ORACLE / TEST INFRASTRUCTURE ONLY.
#
# Builds the reference SU2DMRG (C++/OpenMP) from its own sources into
# oracle/_ref/:
#   oracle/_ref/main_omp       the reference driver, unmodified apart from the
#                              missing-return patch (patch_ref.py)
#   oracle/_ref/libsu2ref.so   the reference objects + harness.cpp, a C entry
#                              layer used to generate golden fixtures
#   oracle/_ref/libsu2ref_mea.so  the same with the engine's measurement
#                              variant (dmrg_su2_omp_mea_enr.cpp) in place of
#                              dmrg_su2_omp.cpp
# The sources are read from $SU2REF_SRC, by default the read-only reference
# checkout this recipe was written against.
# Sources are copied to a scratch directory under /tmp and patched there; the
# reference tree is never written and no reference source enters the repo.
# BLAS/LAPACK come from SciPy's bundled OpenBLAS (blas_shim.c), the Fortran
# helpers from ../fhelpers.c, and mkl.h/mpi.h from shim/.
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REPO="$(cd "$HERE/../.." && pwd)"
SRC="${SU2REF_SRC:-/root/reference}"
OUT="$REPO/oracle/_ref"
if [ ! -f "$SRC/tensor_su2.cpp" ]; then
  # --if-present: a machine without the reference sources (the GPU hosts)
  # uses the committed fixtures instead; nothing to build there
  if [ "${1:-}" = "--if-present" ]; then exit 0; fi
  if [ "${1:-}" = "--shim-check" ]; then exit 77; fi
  echo "build_ref.sh: reference sources not found at $SRC (set SU2REF_SRC)" >&2
  exit 2
fi
# --shim-check: compile include/su2g_tensor_su2_shim.hpp (the binding a
# maintainer adds to the reference tree) against the reference's own headers
if [ "${1:-}" = "--shim-check" ]; then
  CHK="$(mktemp -d /tmp/su2shim.XXXXXX)"
  trap 'rm -rf "$CHK"' EXIT
  echo '#include "su2g_tensor_su2_shim.hpp"' > "$CHK/shim_check.cpp"
  g++ -std=c++17 -fsyntax-only -Wall -I "$SRC" -I "$REPO/include" -I /usr/local/cuda/include "$CHK/shim_check.cpp"
  exit $?
fi
WORK="$(mktemp -d /tmp/su2ref.XXXXXX)"
trap 'rm -rf "$WORK"' EXIT
cp "$SRC"/*.cpp "$SRC"/*.hpp "$WORK"/
python3 "$HERE/patch_ref.py" "$WORK"
OPENBLAS="$(python3 -c 'import scipy,os,glob; d=os.path.join(os.path.dirname(scipy.__file__),"..","scipy.libs"); print(os.path.realpath(sorted(glob.glob(os.path.join(d,"libscipy_openblas*.so")))[0]))')"
OBDIR="$(dirname "$OPENBLAS")"
mkdir -p "$OUT"
CXXFLAGS="-O2 -fopenmp -fPIC -w -I$HERE/shim -I$WORK"
OBJS=()
for f in tensor tensor_dmrg_src tensor_su2 tensor_su2_dmrg_src tensor_su2_hamiltonian \
         su2bond su2struct dmrg_su2 dmrg_su2_omp lanczos_su2; do
  g++ $CXXFLAGS -c "$WORK/$f.cpp" -o "$WORK/$f.o" &
  OBJS+=("$WORK/$f.o")
done
g++ $CXXFLAGS -c "$WORK/main_omp.cpp" -o "$WORK/main_omp.o" &
g++ $CXXFLAGS -c "$HERE/harness.cpp" -o "$WORK/harness.o" &
g++ $CXXFLAGS -c "$WORK/dmrg_su2_omp_mea_enr.cpp" -o "$WORK/dmrg_su2_omp_mea_enr.o" &
g++ $CXXFLAGS -DSU2REF_MEA -c "$HERE/harness.cpp" -o "$WORK/harness_mea.o" &
gcc -O2 -fPIC -c "$REPO/oracle/fhelpers.c" -o "$WORK/fhelpers.o" &
gcc -O2 -fPIC -c "$HERE/blas_shim.c" -o "$WORK/blas_shim.o" &
for job in $(jobs -p); do wait "$job"; done
LIBS=("$WORK/fhelpers.o" "$WORK/blas_shim.o" "$OPENBLAS" -Wl,-rpath,"$OBDIR" -fopenmp)
g++ -o "$OUT/main_omp" "$WORK/main_omp.o" "${OBJS[@]}" "${LIBS[@]}"
g++ -shared -o "$OUT/libsu2ref.so" "$WORK/harness.o" "${OBJS[@]}" "${LIBS[@]}"
# the measurement variant of the engine (dmrg_su2_omp_mea_enr.cpp in place of
# dmrg_su2_omp.cpp), for the centre-bond energy mea_enr
MEA_OBJS=()
for o in "${OBJS[@]}"; do
  if [ "$o" = "$WORK/dmrg_su2_omp.o" ]; then MEA_OBJS+=("$WORK/dmrg_su2_omp_mea_enr.o"); else MEA_OBJS+=("$o"); fi
done
g++ -shared -o "$OUT/libsu2ref_mea.so" "$WORK/harness_mea.o" "${MEA_OBJS[@]}" "${LIBS[@]}"
echo "built $OUT/main_omp, $OUT/libsu2ref.so and $OUT/libsu2ref_mea.so"
