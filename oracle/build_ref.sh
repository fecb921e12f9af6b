#!/bin/sh
# Compiles the reference's own solver templates (from the PASC_inference tree, unmodified)
# together with the shims in oracle/ref_shim into oracle/_ref/libpasc_ref.so.
# Test infrastructure: the library checks the oracle and generates tests/golden/.
# Needs the reference tree at $PASC_REFERENCE (default /root/reference); exits 0 without
# building anything when it is absent.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${PASC_REFERENCE:-/root/reference}
if [ ! -f "$REF/include/general/solver/spgqpsolver.h" ]; then
    echo "build_ref: reference tree not found at $REF; skipped"
    exit 0
fi
mkdir -p "$HERE/_ref"
${CXX:-g++} -std=c++14 -O2 -fPIC -shared -ffp-contract=off -w \
    -I "$HERE/ref_shim" -I "$REF/include" \
    "$HERE/ref_shim/ref_driver.cpp" \
    "$REF/src/general/solver/spg_fs.cpp" \
    "$REF/src/general/solver/generalsolver.cpp" \
    "$REF/src/general/data/generaldata.cpp" \
    "$REF/src/general/model/generalmodel.cpp" \
    -o "$HERE/_ref/libpasc_ref.so"
echo "build_ref: $HERE/_ref/libpasc_ref.so"
