#!/bin/sh
# Regenerate muon.pumas and tau.pumas (the physics dumps shipped with the
# package) from materials.xml with the reference library's
# pumas_physics_create.
# Needs the reference sources (REFERENCE, default: a directory named
# "reference" beside this repository).
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REFERENCE=${REFERENCE:-$(cd "$HERE/../../.." && pwd)/reference}
BUILD="$HERE/_build"
cc -O3 -std=c99 -ffp-contract=off -I"$REFERENCE/include" \
    -o "$BUILD/make_physics" "$HERE/make_physics.c" "$REFERENCE/src/pumas.c" -lm
# The dump records its energy loss directory: muons keep "dedx".
for particle in muon tau; do
        dedx="$BUILD/dedx"
        [ "$particle" = muon ] || dedx="$BUILD/dedx-$particle"
        mkdir -p "$dedx"
        "$BUILD/make_physics" "$HERE/materials.xml" "$dedx" \
            "$BUILD/$particle.pumas" "$particle"
        gzip -9 -n -c "$BUILD/$particle.pumas" > "$HERE/$particle.pumas.gz"
        echo "wrote $HERE/$particle.pumas.gz"
done
