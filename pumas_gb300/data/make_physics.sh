#!/bin/sh
# Regenerate muon.pumas (the physics dump shipped with the package) from
# materials.xml with the reference library's pumas_physics_create.
# Needs the reference sources (REFERENCE, default /root/reference).
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REFERENCE=${REFERENCE:-/root/reference}
BUILD="$HERE/_build"
mkdir -p "$BUILD/dedx"
cc -O3 -std=c99 -ffp-contract=off -I"$REFERENCE/include" \
    -o "$BUILD/make_physics" "$HERE/make_physics.c" "$REFERENCE/src/pumas.c" -lm
"$BUILD/make_physics" "$HERE/materials.xml" "$BUILD/dedx" "$BUILD/muon.pumas"
gzip -9 -n -c "$BUILD/muon.pumas" > "$HERE/muon.pumas.gz"
echo "wrote $HERE/muon.pumas.gz"
