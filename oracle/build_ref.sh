#!/usr/bin/env bash
# Build oracle/_ref/libstref.so from the reference's own tracking sources.
#
# TEST INFRASTRUCTURE ONLY.  The reference's hot path is header-only C; it is
# compiled where it lies (REF_ROOT, default /root/reference) together with
# oracle/ref_driver.c.  The reference normally generates three small
# configuration headers with CMake; this script writes its own versions with
# the reference's default feature values (BB4D/BB6D/SC enabled, TriCub
# disabled, global aperture |x|,|y| < 1 m after every drift) into
# oracle/_ref/include instead of running the reference's build system.
# Flags follow the reference CPU build: -O2 -fno-fast-math, plus
# -ffp-contract=off so no FMA contraction happens on any host.
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF_ROOT="${REF_ROOT:-/root/reference}"
OUT="$HERE/_ref"
if [ ! -f "$REF_ROOT/sixtracklib/common/track/track.h" ]; then
    echo "reference sources not found under $REF_ROOT" >&2
    exit 2
fi
GEN="$OUT/include/sixtracklib/common/generated"
mkdir -p "$GEN"
cat > "$GEN/config.h" <<'EOF'
#ifndef STG_REF_GENERATED_CONFIG_H
#define STG_REF_GENERATED_CONFIG_H
#define SIXTRL_TRACK_MAP_ENABLED 2
#define SIXTRL_TRACK_MAP_SKIP 1
#define SIXTRL_TRACK_MAP_DISABLED 0
#define SIXTRL_TRACK_BEAMBEAM4D 2
#define SIXTRL_TRACK_BEAMBEAM6D 2
#define SIXTRL_TRACK_SPACECHARGE 2
#define SIXTRL_TRACK_TRICUB 0
#define SIXTRL_GLOBAL_APERTURE_CHECK_ALWAYS 2
#define SIXTRL_GLOBAL_APERTURE_CHECK_CONDITIONAL 1
#define SIXTRL_GLOBAL_APERTURE_CHECK_NEVER 0
#define SIXTRL_APERTURE_CHECK_AT_DRIFT 2
#define SIXTRL_APERTURE_CHECK_MIN_DRIFT_LENGTH 0.0
#define SIXTRL_APERTURE_X_LIMIT 1.0
#define SIXTRL_APERTURE_Y_LIMIT 1.0
#endif
EOF
cat > "$GEN/namespace.h" <<'EOF'
#ifndef STG_REF_GENERATED_NAMESPACE_H
#define STG_REF_GENERATED_NAMESPACE_H
#define SIXTRL_C99_NAMESPACE st_
#define SIXTRL_C99_NAMESPACE_STR "st_"
#define SIXTRL_C99_NAMESPACE_PREFIX_STR "st_"
#define SIXTRL_CXX_NAMESPACE sixtrack
#define SIXTRL_CXX_NAMESPACE_STR "sixtrack"
#define SIXTRL_CXX_NAMESPACE_PREFIX_STR "sixtrack::"
#endif
EOF
cat > "$GEN/modules.h" <<'EOF'
#ifndef STG_REF_GENERATED_MODULES_H
#define STG_REF_GENERATED_MODULES_H
#define SIXTRACKLIB_ENABLE_MODULE_SIMD 0
#define SIXTRACKLIB_ENABLE_MODULE_OPENCL 0
#define SIXTRACKLIB_ENABLE_MODULE_CUDA 0
#define SIXTRACKLIB_ENABLE_MODULE_MPFR4 0
#endif
EOF
CFLAGS="-O2 -fPIC -std=gnu99 -fno-fast-math -ffp-contract=off -DNDEBUG -w"
gcc $CFLAGS -shared -I "$OUT/include" -I "$REF_ROOT" -I "$HERE" \
    "$HERE/ref_driver.c" -o "$OUT/libstref.so" -lm
# The per-particle OpenMP baseline driver (same reference function per
# particle, parallel over particles), used for CPU timing here.
gcc $CFLAGS -fopenmp -shared -I "$OUT/include" -I "$REF_ROOT" -I "$HERE" \
    "$HERE/ref_driver.c" -DSTG_REF_OMP -o "$OUT/libstref_omp.so" -lm
echo "built $OUT/libstref.so"
