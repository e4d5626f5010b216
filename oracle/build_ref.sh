#!/usr/bin/env bash
# Builds the reference VariantDBSCAN CPU library (the checker, never the product)
# into oracle/_ref/libSharedVDBSCAN.so.
#
# Recipe:
#   1. When VDB_REFERENCE_DIR names a checkout of the reference, stage its CPU
#      sources (src/*.cpp, src/*.h of the libSharedVDBSCAN target,
#      src/makefile:25-35) into oracle/_ref/src/, and the unmodified callers
#      of its C ABI that the drop-in tests build against the GB300 library
#      (src/c_test_prog.{cpp,h} with its fixture src/test_dataset.csv, and the
#      Python wrapper python_package/vdbscan/variantdbscan.py) into
#      oracle/_ref/callers/.  The staged copies are build intermediates:
#      oracle/_ref/ is git-ignored.
#   2. Apply the one-line build fix to the staged DBScan.cpp: the reference
#      declares `int DBScan::filterCandidatesMPB(...)` (src/DBScan.cpp:665) and
#      falls off its end (src/DBScan.cpp:695).  GCC >= 8 treats that as
#      unreachable and drops the candidate loop's exit, so the library crashes
#      as shipped.  The fix inserts `return 0;` before the closing brace; the
#      return value is ignored by the only caller (src/DBScan.cpp:656), so the
#      results are unchanged.
#   3. Compile the staged sources with g++ -O3 -fopenmp and
#      -ffp-contract=off (the reference was built for x86-64, where GCC has no
#      FMA to contract into; on aarch64 GCC would otherwise fuse the distance
#      arithmetic of src/DBScan.cpp:701 and change boundary pairs).
#
# Without VDB_REFERENCE_DIR (e.g. on a machine that only received the staged
# copy), step 3 runs on oracle/_ref/src/ if it exists.
set -euo pipefail

HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
OUT="$HERE/_ref"
SRC="$OUT/src"
REF="${VDB_REFERENCE_DIR:-}"
NTHREADS="${VDB_REF_THREADS:-$(nproc)}"
CXX="${CXX:-g++}"

FILES="DBScan.cpp DBScan.h main.cpp schedule.cpp schedule.h tree_functions.cpp structs.h globals.h prototypes.h RTree.h"

mkdir -p "$SRC"
if [ -n "$REF" ] && [ -d "$REF/src" ]; then
  for f in $FILES; do
    cp "$REF/src/$f" "$SRC/$f"
  done
  mkdir -p "$OUT/callers"
  for f in c_test_prog.cpp c_test_prog.h test_dataset.csv test_output.csv; do
    cp "$REF/src/$f" "$OUT/callers/$f"
  done
  cp "$REF/python_package/vdbscan/variantdbscan.py" "$OUT/callers/variantdbscan.py"
  # the closing brace of filterCandidatesMPB must be line 695
  if [ "$(sed -n '695p' "$SRC/DBScan.cpp" | tr -d '[:space:]')" != "}" ]; then
    echo "build_ref.sh: unexpected DBScan.cpp layout at line 695" >&2
    exit 1
  fi
  sed -i '695i\		return 0;' "$SRC/DBScan.cpp"
fi

if [ ! -f "$SRC/DBScan.cpp" ]; then
  echo "build_ref.sh: no reference sources (set VDB_REFERENCE_DIR)" >&2
  exit 2
fi

FLAGS="-O3 -fopenmp -fPIC -ffp-contract=off -DNSEARCHTHREADS=$NTHREADS -w"
pids=""
for f in main schedule DBScan tree_functions; do
  "$CXX" $FLAGS -c "$SRC/$f.cpp" -o "$OUT/$f.o" &
  pids="$pids $!"
done
for p in $pids; do wait "$p"; done
"$CXX" -O3 -shared -fopenmp -fPIC "$OUT/main.o" "$OUT/schedule.o" "$OUT/DBScan.o" \
  "$OUT/tree_functions.o" -o "$OUT/libSharedVDBSCAN.so"
echo "$NTHREADS" > "$OUT/NSEARCHTHREADS"
echo "built $OUT/libSharedVDBSCAN.so (NSEARCHTHREADS=$NTHREADS)"
