#!/bin/sh
# Compiles the reference's own DSGL trainer -- include/dsgl.hpp of trsenli/GDistGER-re,
# read in place and unmodified -- against the single-rank MPI and cblas stand-ins in
# oracle/ref_shim, into oracle/_ref/dsgl_ref.  Test infrastructure only (the golden
# vectors of tests/golden/ come from this binary).
#
# The reference checkout is REF_ROOT; unset, the recipe looks where the build container
# keeps the read-only checkout, /root/reference (this recipe is the one place that names
# it).  With --if-present a missing checkout is not an error (GPU hosts have none).
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${REF_ROOT:-/root/reference}
if [ ! -f "$REF/include/dsgl.hpp" ]; then
  if [ "$1" = "--if-present" ]; then
    echo "reference sources not found under $REF: harness not built"
    exit 0
  fi
  echo "reference sources not found under $REF (set REF_ROOT)" >&2
  exit 1
fi
mkdir -p "$HERE/_ref"
g++ -O3 -std=c++14 -fopenmp -ffp-contract=off -DUSE_MKL -w \
    -I "$HERE/ref_shim" -I "$REF/include" \
    "$HERE/ref_driver.cpp" -o "$HERE/_ref/dsgl_ref"
echo "built $HERE/_ref/dsgl_ref"
