#!/bin/sh
# Builds the reference drivers of oracle/_ref/ from LMT++'s own sources where they lie (read-only):
#   ref_codegen  - LMT++'s symbolic engine (include/codegen) driven on the weak forms of the hot
#                  path; run here, it writes the element routines it emits (_ref/gen_elem.h,
#                  gen_elem.cpp, gen_recal.cpp);
#   ref_driver   - LMT++'s runtime (make_rect, Sym SparseLine assembly, penalty, LDL, IC(0)-PCG,
#                  3x3-block IC-PCG) around those routines;
#   ref_meshio, ref_vtu_elast - LMT++'s mesh reader and VTU writer.
# Test infrastructure only; outputs go to oracle/_ref/.  The recipe reads the LMTpp sources at
# $LMTPP_SRC (default /root/reference) and skips everything when they are absent.
set -e
HERE="$(cd "$(dirname "$0")" && pwd)"
SRC="${LMTPP_SRC:-/root/reference}"
OUT="$HERE/_ref"
if [ ! -d "$SRC/include" ]; then
  echo "build_ref: no LMTpp sources at $SRC, skipping" >&2
  exit 0
fi
# up to date: every driver newer than this recipe and the oracle's C++ sources
if [ -x "$OUT/ref_driver" ] && [ -x "$OUT/ref_meshio" ] && [ -x "$OUT/ref_vtu_elast" ] && [ -z "$LMTG_REF_FORCE" ] &&
   [ -z "$(find "$HERE" -maxdepth 1 \( -name 'ref_*.cpp' -o -name build_ref.sh \) -newer "$OUT/ref_driver")" ]; then
  echo "build_ref: up to date"
  exit 0
fi
mkdir -p "$OUT/obj" "$OUT/cg"
echo "$SRC" > "$OUT/lmtpp_src"  # where the sources were found, for the adapter's compile test
CFLAGS="-O2 -w -DDINT -DDONT_WANT_XML"
RFLAGS="$CFLAGS -std=gnu++98 -fpermissive -I$SRC/include -I$SRC/include/amd -I$SRC/include/LDL"
for f in "$SRC"/include/amd/amd_*.c; do
  b=$(basename "$f" .c)
  gcc $CFLAGS -I"$SRC/include/amd" -c "$f" -o "$OUT/obj/$b.o" &
done
g++ $CFLAGS -x c++ -I"$SRC/include/amd" -I"$SRC/include/LDL" -c "$SRC/include/LDL/ldl.cpp" -o "$OUT/obj/ldl.o" &
g++ $RFLAGS -c "$SRC/include/util/solveLDL.cpp" -o "$OUT/obj/solveLDL.o" &
g++ $RFLAGS -c "$SRC/include/util/solveLDL_semimorse.cpp" -o "$OUT/obj/solveLDL_semimorse.o" &
# the symbolic engine (exsolver.cpp needs GSL and is not on this path)
for f in ex op exvector exmatrix read_ex write_code write_code_language_cpp write_graphviz; do
  g++ $CFLAGS -std=gnu++98 -fpermissive -I"$SRC/include/codegen" -c "$SRC/include/codegen/$f.cpp" -o "$OUT/cg/$f.o" &
done
g++ $CFLAGS -std=gnu++98 -fpermissive -I"$SRC/include" "$HERE/ref_meshio.cpp" -o "$OUT/ref_meshio" &
g++ $CFLAGS -std=gnu++98 -fpermissive -I"$SRC/include" "$HERE/ref_vtu_elast.cpp" -o "$OUT/ref_vtu_elast" &
wait
g++ $CFLAGS -std=gnu++98 -fpermissive -I"$SRC/include/codegen" "$HERE/ref_codegen.cpp" "$OUT"/cg/*.o -o "$OUT/ref_codegen"
"$OUT/ref_codegen" "$OUT/gen_elem.h" "$OUT/gen_elem.cpp" "$OUT/gen_recal.cpp"
# the recalage routines are straight-line functions of tens of thousands of terms, which the
# optimiser takes hours over: they build at -O0 (IEEE double arithmetic either way)
g++ -O2 -w -I"$OUT" -c "$OUT/gen_elem.cpp" -o "$OUT/obj/gen_elem.o" &
g++ -O0 -w -I"$OUT" -c "$OUT/gen_recal.cpp" -o "$OUT/obj/gen_recal.o" &
g++ $RFLAGS -I"$OUT" -c "$HERE/ref_driver.cpp" -o "$OUT/obj/ref_driver.o" &
wait
g++ -o "$OUT/ref_driver" "$OUT"/obj/*.o -lpthread
echo "build_ref: $OUT/ref_driver $OUT/ref_meshio $OUT/ref_vtu_elast (element routines: $OUT/gen_elem.cpp, $OUT/gen_recal.cpp)"
