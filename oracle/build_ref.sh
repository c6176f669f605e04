#!/bin/sh
# Recipe: builds oracle/_ref/libftref.so from the reference's own
# sodium_fe.cu / sodium_ge.cu (host-compiled, CUDA qualifiers defined away),
# read where they lie.  FT_REF_SRC names the reference's src/ directory; the
# default is the read-only checkout of the development container.  Does
# nothing (exit 0) where the sources are absent, as on the GPU host.
#   sh oracle/build_ref.sh          build
#   sh oracle/build_ref.sh --src    print the source directory and exit
set -e
REF_SRC="${FT_REF_SRC:-/root/reference/src}"
if [ "$1" = "--src" ]; then
    echo "$REF_SRC"
    exit 0
fi
HERE="$(cd "$(dirname "$0")" && pwd)"
if [ ! -f "$REF_SRC/sodium_fe.cu" ]; then
    echo "reference sources not found at $REF_SRC; skipping oracle/_ref" >&2
    exit 0
fi
mkdir -p "$HERE/_ref"
g++ -O2 -fPIC -shared -x c++ -D__host__= -D__device__= -D__global__= \
    -I"$REF_SRC" -w -o "$HERE/_ref/libftref.so" "$HERE/ref_shim.cc"
echo "built $HERE/_ref/libftref.so"
