#!/bin/sh
# Builds oracle/_ref/ref_driver from the reference's own sources where they lie (read-only),
# plus the oracle's element integrand.  Test infrastructure only; outputs go to oracle/_ref/.
# Needs the LMTpp sources at $LMTPP_SRC (default /root/reference); skipped when absent.
set -e
HERE="$(cd "$(dirname "$0")" && pwd)"
SRC="${LMTPP_SRC:-/root/reference}"
OUT="$HERE/_ref"
if [ ! -d "$SRC/include" ]; then
  echo "build_ref: no LMTpp sources at $SRC, skipping" >&2
  exit 0
fi
mkdir -p "$OUT/obj"
CFLAGS="-O2 -w -DDINT -DDONT_WANT_XML"
for f in "$SRC"/include/amd/amd_*.c; do
  b=$(basename "$f" .c)
  gcc $CFLAGS -I"$SRC/include/amd" -c "$f" -o "$OUT/obj/$b.o" &
done
g++ $CFLAGS -x c++ -I"$SRC/include/amd" -I"$SRC/include/LDL" -c "$SRC/include/LDL/ldl.cpp" -o "$OUT/obj/ldl.o" &
g++ $CFLAGS -std=gnu++98 -fpermissive -I"$SRC/include" -I"$SRC/include/amd" -I"$SRC/include/LDL" \
    -c "$SRC/include/util/solveLDL.cpp" -o "$OUT/obj/solveLDL.o" &
g++ $CFLAGS -std=gnu++98 -fpermissive -I"$SRC/include" -I"$SRC/include/amd" -I"$SRC/include/LDL" \
    -c "$SRC/include/util/solveLDL_semimorse.cpp" -o "$OUT/obj/solveLDL_semimorse.o" &
gcc -O2 -std=c99 -c "$HERE/fe_oracle.c" -o "$OUT/obj/fe_oracle.o" &
g++ $CFLAGS -std=gnu++98 -fpermissive -I"$SRC/include" -I"$SRC/include/amd" -I"$SRC/include/LDL" -I"$HERE" \
    -c "$HERE/ref_driver.cpp" -o "$OUT/obj/ref_driver.o" &
g++ $CFLAGS -std=gnu++98 -fpermissive -I"$SRC/include" "$HERE/ref_meshio.cpp" -o "$OUT/ref_meshio" &
g++ $CFLAGS -std=gnu++98 -fpermissive -I"$SRC/include" "$HERE/ref_vtu_elast.cpp" -o "$OUT/ref_vtu_elast" &
wait
g++ -o "$OUT/ref_driver" "$OUT"/obj/*.o -lpthread
echo "build_ref: $OUT/ref_driver $OUT/ref_meshio $OUT/ref_vtu_elast"
