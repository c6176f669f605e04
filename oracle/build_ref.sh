#!/bin/sh
# Builds oracle/_ref/libftref.so from the reference's own sodium_fe.cu /
# sodium_ge.cu (host-compiled, CUDA qualifiers defined away).  Needs the
# reference source tree; does nothing (exit 0) where it is absent.
set -e
REF_SRC="${FT_REF_SRC:-/root/reference/src}"
HERE="$(cd "$(dirname "$0")" && pwd)"
if [ ! -f "$REF_SRC/sodium_fe.cu" ]; then
    echo "reference sources not found at $REF_SRC; skipping oracle/_ref" >&2
    exit 0
fi
mkdir -p "$HERE/_ref"
g++ -O2 -fPIC -shared -x c++ -D__host__= -D__device__= -D__global__= \
    -I"$REF_SRC" -w -o "$HERE/_ref/libftref.so" "$HERE/ref_shim.cc"
echo "built $HERE/_ref/libftref.so"
