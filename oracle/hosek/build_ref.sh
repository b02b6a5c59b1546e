#!/bin/sh
# Builds oracle/_ref/hosek_ref from the reference's own sources where they lie
# (evaluate_spline/evaluate of src/engine/gfx/hosek_wilkie_sky_model.cpp:41-67
# and include/gfx/hosek_data_rgb.inl) and regenerates the derived table and
# the golden fixture.  Needs the reference tree, named by $HELIOS_REFERENCE;
# run from the repository root.
set -e
REF=${HELIOS_REFERENCE:?set HELIOS_REFERENCE to the reference tree}
mkdir -p oracle/_ref
sed -n '41,67p' "$REF/src/engine/gfx/hosek_wilkie_sky_model.cpp" > oracle/_ref/hw_eval_ref.inc
g++ -O2 -std=c++17 -ffp-contract=off -I oracle/_ref -I "$REF/include/gfx" \
    -o oracle/_ref/hosek_ref oracle/hosek/hosek_ref_main.cpp
./oracle/_ref/hosek_ref helios_gb300/csrc/hosek_table.inc tests/golden/hosek_coeffs.json
