#!/bin/sh
# Compiles the reference's own solver templates (from the PASC_inference tree, unmodified)
# together with the shims in oracle/ref_shim into oracle/_ref/libpasc_ref.so.
# Test infrastructure: the library checks the oracle and generates tests/golden/.
# Needs the reference tree at $PASC_REFERENCE (default /root/reference); exits 0 without
# building anything when it is absent (pasc_oracle.build_ref then compiles the flattened
# translation unit this recipe left in oracle/_ref, if there is one).
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${PASC_REFERENCE:-/root/reference}
if [ ! -f "$REF/include/general/solver/spgqpsolver.h" ]; then
    echo "build_ref: reference tree not found at $REF; skipped"
    exit 0
fi
mkdir -p "$HERE/_ref"
${CXX:-g++} -std=c++14 -O2 -fopenmp -fPIC -shared -ffp-contract=off -w \
    -I "$HERE/ref_shim" -I "$REF/include" \
    "$HERE/ref_shim/ref_driver.cpp" \
    "$REF/src/general/solver/spg_fs.cpp" \
    "$REF/src/general/solver/generalsolver.cpp" \
    "$REF/src/general/data/generaldata.cpp" \
    "$REF/src/general/model/generalmodel.cpp" \
    -o "$HERE/_ref/libpasc_ref.so"
echo "build_ref: $HERE/_ref/libpasc_ref.so"
# The same library as one translation unit (reference headers and sources, shims inlined), so
# that pasc_oracle.build_ref() can compile it where the reference tree is absent.
python3 "$HERE/flatten_sources.py" "$HERE/_ref/libpasc_ref_flat.cpp" \
    "$HERE/ref_shim/ref_driver.cpp" \
    "$REF/src/general/solver/spg_fs.cpp" \
    "$REF/src/general/solver/generalsolver.cpp" \
    "$REF/src/general/data/generaldata.cpp" \
    "$REF/src/general/model/generalmodel.cpp" \
    -I "$HERE/ref_shim" -I "$REF/include" -I "$REF/src"
echo "build_ref: $HERE/_ref/libpasc_ref_flat.cpp"
# The test driver of the GB300 backend (tests/cpp/gb300_backend_driver.cpp, include/pasc/
# gb300_backend.hpp) over the reference's generic solver templates, as one translation unit
# with the reference's headers and the shims inlined (this repository's headers stay
# includes), for tests/test_gpu_backend.py to compile where the reference tree is absent.
ROOT=$(cd "$HERE/.." && pwd)
python3 "$HERE/flatten_sources.py" "$HERE/_ref/backend/gb300_backend_driver_flat.cpp" \
    "$ROOT/tests/cpp/gb300_backend_driver.cpp" \
    "$REF/src/general/solver/spg_fs.cpp" \
    "$REF/src/general/solver/generalsolver.cpp" \
    "$REF/src/general/data/generaldata.cpp" \
    "$REF/src/general/model/generalmodel.cpp" \
    -I "$HERE/ref_shim" -I "$REF/include" -I "$REF/src"
echo "build_ref: $HERE/_ref/backend/gb300_backend_driver_flat.cpp"
