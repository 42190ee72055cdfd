#!/bin/sh
# Builds the reference's own hot-path sources into oracle/_ref/ (git-ignored).
# TEST INFRASTRUCTURE ONLY: the result pins the oracle restatement and makes
# the golden fixtures; the product never links it.
#
# The sources are compiled where they lie, read-only, with the reference's
# own release flags (ClusteredCore/Release/src/subdir.mk: -std=c++0x -O3
# -fopenmp -fPIC) plus -ffp-contract=off so that no host contracts a*b+c.
# The prebuilt binaries shipped inside the reference tree are never used.
#   libpsimref.so      ClusteredCore (minus fastRandom.cpp, replaced by the
#                      noise-injection shim) + AOPotential + LennardJones +
#                      Calibration (factories renamed by -DgetForce=...) +
#                      ref_harness.cpp
#   libpsimref_rng.so  ClusteredCore with the real fastRandom.cpp + ref_rng.cpp
set -e
REF=${PSIM_REFERENCE:-/root/reference}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
if [ ! -d "$REF/ClusteredCore/src" ]; then
    echo "reference sources not found at $REF; oracle/_ref not built" >&2
    exit 3
fi
CXX=${CXX:-g++}
FLAGS="-std=c++0x -O3 -fopenmp -fPIC -ffp-contract=off -w"
INC="-I$REF/ClusteredCore/include"
mkdir -p "$OUT/obj"

pids=""
for src in $(find "$REF/ClusteredCore/src" -name '*.cpp' | sort); do
    base=$(basename "$src" .cpp)
    $CXX $FLAGS $INC -c "$src" -o "$OUT/obj/core_$base.o" &
    pids="$pids $!"
done
$CXX $FLAGS $INC -I"$REF/AOPotential/include" -DgetForce=psimref_getForce_AO \
    -c "$REF/AOPotential/src/AOPotential.cpp" -o "$OUT/obj/plugin_AO.o" &
pids="$pids $!"
$CXX $FLAGS $INC -I"$REF/LennardJones/include" -DgetForce=psimref_getForce_LJ \
    -c "$REF/LennardJones/src/LJPotential.cpp" -o "$OUT/obj/plugin_LJ.o" &
pids="$pids $!"
$CXX $FLAGS $INC -I"$REF/Calibration/include" -DgetForce=psimref_getForce_Cal \
    -c "$REF/Calibration/src/Calibration.cpp" -o "$OUT/obj/plugin_Cal.o" &
pids="$pids $!"
$CXX $FLAGS $INC -c "$HERE/ref_noise_shim.cpp" -o "$OUT/obj/shim.o" &
pids="$pids $!"
$CXX $FLAGS $INC -c "$HERE/ref_harness.cpp" -o "$OUT/obj/harness.o" &
pids="$pids $!"
$CXX $FLAGS $INC -c "$HERE/ref_rng.cpp" -o "$OUT/obj/rng.o" &
pids="$pids $!"
for p in $pids; do wait "$p"; done

CORE=$(ls "$OUT"/obj/core_*.o | grep -v core_fastRandom.o)
$CXX -shared -fopenmp -o "$OUT/libpsimref.so" $CORE "$OUT/obj/shim.o" \
    "$OUT/obj/plugin_AO.o" "$OUT/obj/plugin_LJ.o" "$OUT/obj/plugin_Cal.o" \
    "$OUT/obj/harness.o"
$CXX -shared -fopenmp -o "$OUT/libpsimref_rng.so" $CORE "$OUT/obj/core_fastRandom.o" \
    "$OUT/obj/rng.o"
echo "built $OUT/libpsimref.so $OUT/libpsimref_rng.so"
