#!/bin/sh
# Installs the reference ODP library's own C/CUDA sources and its sample
# programs into baseline/_ref/src
# (git-ignored), so that they travel with the working tree to machines where
# the reference tree itself is absent.  `pip install` cannot do this: the
# reference is a C project with neither setup.py nor pyproject.toml.
#
#   sh baseline/install_ref.sh [REFERENCE_DIR]
#
# REFERENCE_DIR defaults to $ODP_REFERENCE_DIR, else /root/reference.  The
# files are copied unmodified; nothing here is committed.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
SRC=${1:-${ODP_REFERENCE_DIR:-/root/reference}}
DST="$HERE/_ref/src"
if [ ! -f "$SRC/aspl.c" ] || [ ! -f "$SRC/include/odp.h" ]; then
  echo "install_ref.sh: no reference tree at $SRC" >&2
  exit 1
fi
mkdir -p "$DST/include"
for f in aspl.c utils.c aspl_cuda.cu utils_cuda.cu common.h parameter.h LICENSE; do
  cp -p "$SRC/$f" "$DST/$f"
done
cp -p "$SRC/include/odp.h" "$DST/include/odp.h"
# the sample programs and their golden tables (sample/Makefile's test data)
rm -rf "$DST/sample"
cp -pR "$SRC/sample" "$DST/sample"
echo "reference sources installed in $DST"
