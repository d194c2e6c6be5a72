#!/bin/sh
# Compiles the reference's own DSGL trainer -- include/dsgl.hpp of trsenli/GDistGER-re,
# read in place and unmodified -- against the single-rank MPI and cblas stand-ins in
# oracle/ref_shim, into oracle/_ref/dsgl_ref.  Test infrastructure only (the golden
# vectors of tests/golden/ come from this binary).  Needs the reference checkout.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${REF_ROOT:-/root/reference}
if [ ! -f "$REF/include/dsgl.hpp" ]; then
  echo "reference sources not found under $REF" >&2
  exit 1
fi
mkdir -p "$HERE/_ref"
g++ -O3 -std=c++14 -fopenmp -ffp-contract=off -DUSE_MKL -w \
    -I "$HERE/ref_shim" -I "$REF/include" \
    "$HERE/ref_driver.cpp" -o "$HERE/_ref/dsgl_ref"
echo "built $HERE/_ref/dsgl_ref"
