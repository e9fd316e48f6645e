#!/bin/sh
# Build the unmodified reference C model with oracle/ref_shim.cpp into oracle/_ref/cmodel_ref.
# Reads the reference sources where they lie; writes only under oracle/_ref/.  Exits 0 without
# building when the reference tree is not present (it exists only where the reference is mounted).
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
SRC=${MDRL_REFERENCE:-/root/reference}/Range_Limited_demo/SourceCode/C_Model_ForceEval/MD_Evaluation_Model.cpp
if [ ! -f "$SRC" ]; then
    echo "reference C model not present; oracle/_ref not built"
    exit 0
fi
mkdir -p "$HERE/_ref"
g++ -O2 -ffp-contract=off -fno-fast-math -rdynamic -o "$HERE/_ref/cmodel_ref" "$SRC" "$HERE/ref_shim.cpp" -ldl
echo "$HERE/_ref/cmodel_ref"
