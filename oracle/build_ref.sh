#!/usr/bin/env bash
# Builds oracle/_ref/librvref.so from RecView's own sources, unmodified, where they lie.
#
# TEST INFRASTRUCTURE ONLY: the library is the parity pin for the oracle restatement
# (oracle/rv_oracle.c) and is used by tests and fixture generation in the container that has
# the reference checkout.  Nothing is copied into the repository: whole files are compiled by
# path, and the function bodies below are spliced between small wrapper heads/tails
# (oracle/ref_wrap) through a pipe straight into the compiler.  Outputs go to oracle/_ref only.
#
#   source/cfft.cpp, source/ccmplx.cpp             compiled by path
#   source/general.cpp:2020-2163                  CPU back-projection body (scalar loop)
#   source/general.cpp:2377-2532                  GenerateSinogramThread
#   source/gazoDoc.cpp:3748-3812                  body of CGazoDoc::SetFilter
#   source/gazoDoc.cpp:4379-4627                  computational part of CGazoDoc::GetAxis
#   source/general.cpp:1313-1470                  WriteTifMonochrome16 (16-bit TIFF writer)
#   source/gazoDoc.cpp:2967-2978, 3535-3666        GetSinogramYdim + offset-CT stitching tail
#   source/gazoDoc.cpp:3002-3004, 3318-3342        strip assembly: trim and bin x bin average
#   oracle/ref_wrap/libm_pin.cpp                  correctly rounded cosf/sinf for the twiddles
#
# The extracted ranges are checked against SHA-256 sums so a different checkout fails loudly
# instead of silently compiling the wrong lines.
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
# The reference checkout: RECVIEW_REFERENCE, else the location this recipe was written for.
SRC="${RECVIEW_REFERENCE:-/root/reference}/source"
OUT="$HERE/_ref"
if [ ! -d "$SRC" ]; then
    echo "build_ref: reference sources not found at $SRC; skipping" >&2
    exit 3
fi
mkdir -p "$OUT/obj" "$OUT/gen"
# source/cfft.cpp:530 includes <sys\timeb.h> with a Windows path separator; on Linux that is a
# file name containing a backslash, generated here (outside the repository's tracked files).
printf '#include <afx.h>\n' > "$OUT/gen/sys\\timeb.h"

check() {  # file first last sha256
    local got
    got="$(sed -n "$2,$3p" "$SRC/$1" | sha256sum | cut -d' ' -f1)"
    if [ "$got" != "$4" ]; then
        echo "build_ref: $1:$2-$3 differs from the audited checkout ($got)" >&2
        exit 4
    fi
}
check general.cpp 2020 2163 0363b3ff22cd95c6b3c1aa74a56ec5eb8c6fd5e225459306ffdbaa97adf2ff28
check general.cpp 2377 2532 2f41a4c98ee29e23f3a3dc7d8e5ddc1289e70dd46e097b141a26bd4c4a033981
check gazoDoc.cpp 3748 3812 74de08b2b13fbf43c047b1fdca2bff6aae955307240a1aed58a8024175e90a3d
check general.cpp 1313 1470 80bb671236c506c654d4f1f620d23d219fa28b59a121d4f25384e6f6054c2c56
check gazoDoc.cpp 4379 4627 fcf94fb4d8af6e867fe5ecef64c6d776047c3b5bea9ea73fa5fd83c00b407774
check gazoDoc.cpp 2967 2978 d0d0a88882e1b0a605ad40cbe58e122756669c99033dbdf55af4b2aceb72b678
check gazoDoc.cpp 3535 3666 20e3f0e0c127d19e8d899301a4ddfc030737579b554f0435a85014666a383e8b
check gazoDoc.cpp 3002 3004 b1dd6f55c31e6bfe54ab82aa991d67f686cd3b7021d472f12f134efadb2bae65
check gazoDoc.cpp 3318 3342 14859f870809e364a7d248be4ea7ffef60de97ccacf31d2285216b9bb517ab18

CXX="${CXX:-g++}"
# -ffp-contract=off: the reference's x64 build rounds every float operation separately.
FLAGS=(-O2 -ffp-contract=off -fPIC -w -fpermissive -I"$HERE/ref_shim" -I"$OUT/gen" -I"$SRC")

cd "$OUT/obj"   # empty directory: quote includes of the piped units resolve via -I only
"$CXX" "${FLAGS[@]}" -c "$SRC/cfft.cpp" -o cfft.o
"$CXX" "${FLAGS[@]}" -c "$SRC/ccmplx.cpp" -o ccmplx.o
{ cat "$HERE/ref_wrap/fbp_head.inc"; sed -n 2020,2163p "$SRC/general.cpp"; cat "$HERE/ref_wrap/fbp_tail.inc"; } \
    | "$CXX" "${FLAGS[@]}" -x c++ -c - -o fbp.o
{ cat "$HERE/ref_wrap/sino_head.inc"; sed -n 2377,2532p "$SRC/general.cpp"; cat "$HERE/ref_wrap/sino_tail.inc"; } \
    | "$CXX" "${FLAGS[@]}" -x c++ -c - -o sino.o
{ cat "$HERE/ref_wrap/filter_head.inc"; sed -n 3748,3812p "$SRC/gazoDoc.cpp"; cat "$HERE/ref_wrap/filter_tail.inc"; } \
    | "$CXX" "${FLAGS[@]}" -x c++ -c - -o filter.o
{ cat "$HERE/ref_wrap/axis_head.inc"; sed -n 4379,4627p "$SRC/gazoDoc.cpp"; cat "$HERE/ref_wrap/axis_tail.inc"; } \
    | "$CXX" "${FLAGS[@]}" -x c++ -c - -o axis.o
{ cat "$HERE/ref_wrap/tif_head.inc"; sed -n 1313,1470p "$SRC/general.cpp"; cat "$HERE/ref_wrap/tif_tail.inc"; } \
    | "$CXX" "${FLAGS[@]}" -x c++ -c - -o tif.o
{ cat "$HERE/ref_wrap/ofct_head.inc"; sed -n 2967,2978p "$SRC/gazoDoc.cpp"; cat "$HERE/ref_wrap/ofct_mid.inc"; \
  sed -n 3535,3666p "$SRC/gazoDoc.cpp"; cat "$HERE/ref_wrap/ofct_tail.inc"; } \
    | "$CXX" "${FLAGS[@]}" -x c++ -c - -o ofct.o
{ cat "$HERE/ref_wrap/bin_head.inc"; sed -n 3002,3004p "$SRC/gazoDoc.cpp"; sed -n 3318,3342p "$SRC/gazoDoc.cpp"; \
  cat "$HERE/ref_wrap/bin_tail.inc"; } \
    | "$CXX" "${FLAGS[@]}" -x c++ -c - -o bin.o
"$CXX" "${FLAGS[@]}" -fno-builtin -c "$HERE/ref_wrap/libm_pin.cpp" -o libm_pin.o
"$CXX" -shared -o "$OUT/librvref.so" cfft.o ccmplx.o fbp.o sino.o filter.o axis.o tif.o ofct.o bin.o libm_pin.o -lm
echo "build_ref: $OUT/librvref.so"
