#!/usr/bin/env bash
# Builds the BlochLib reference's powder-FID path into oracle/_ref/ (git-ignored).
# Test infrastructure only: the binaries are the oracle that pins the CPU restatement
# and the golden FIDs, and the timed CPU baseline.  Nothing here is linked into the
# product.
#
#   ref_fid    the reference as shipped (its QL eigen-iteration runs in float)
#   ref_fid64  the same sources with that iteration in double (the FP64 oracle)
#
# Source: $BLOCHLIB_REF/src (default: the reference tree's mount point below) is copied to oracle/_ref/src
# and build-fixed by patch_ref.py; the propagator-reduction class of the MMMQMAS example
# (examples/qmsims/MMMQMAS/propreduce.{h,cc}) is copied unchanged to oracle/_ref/mmmqmas,
# beside a one-line blochlib.h that includes only QMspins/sys.h (the umbrella header pulls
# in unrelated, unpatched parts of the tree).  Where the reference tree is absent but a
# scratch copy already sits in oracle/_ref, that copy is built as is.
#   usage: build_ref.sh [f32|f64|all]   (default all)
#          build_ref.sh where             prints the reference tree's path (exit 3 if absent)
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
ref="${BLOCHLIB_REF:-/root/reference}"
which="${1:-all}"
if [ "$which" = where ]; then
  if [ -d "$ref/src" ]; then echo "$ref"; exit 0; fi
  exit 3
fi
mkdir -p "$here/_ref"
if [ -d "$ref/src" ]; then
  if [ ! -f "$here/_ref/src/.patched" ] || [ "$here/patch_ref.py" -nt "$here/_ref/src/.patched" ]; then
    rm -rf "$here/_ref/src"
    cp -r "$ref/src" "$here/_ref/src"
    chmod -R u+w "$here/_ref/src"
    python3 "$here/patch_ref.py" "$here/_ref/src"
    touch "$here/_ref/src/.patched"
  fi
  mkdir -p "$here/_ref/mmmqmas"
  for f in propreduce.h propreduce.cc; do
    if [ ! -f "$here/_ref/mmmqmas/$f" ] || [ "$ref/examples/qmsims/MMMQMAS/$f" -nt "$here/_ref/mmmqmas/$f" ]; then
      cp "$ref/examples/qmsims/MMMQMAS/$f" "$here/_ref/mmmqmas/$f"
      chmod u+w "$here/_ref/mmmqmas/$f"
    fi
  done
  printf '#include "QMspins/sys.h"\n' > "$here/_ref/mmmqmas/blochlib.h"
elif [ ! -f "$here/_ref/src/.patched" ]; then
  echo "build_ref.sh: reference sources not found (set BLOCHLIB_REF)" >&2
  exit 3
fi
jobs="$(nproc 2>/dev/null || echo 4)"
cd "$here"
if [ "$which" = all ] || [ "$which" = f32 ]; then
  make -s -j"$jobs" -f ref.mk QL=float BIN=_ref/ref_fid OBJ=_ref/obj_f32
fi
if [ "$which" = all ] || [ "$which" = f64 ]; then
  make -s -j"$jobs" -f ref.mk QL=double BIN=_ref/ref_fid64 OBJ=_ref/obj_f64
fi
