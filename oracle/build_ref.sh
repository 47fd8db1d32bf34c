#!/usr/bin/env bash
# Build oracle/_ref/libstref.so from the reference's own tracking sources.
#
# TEST INFRASTRUCTURE ONLY.  The reference's hot path is header-only C; it is
# compiled where it lies (REF_ROOT, default /root/reference) together with
# oracle/ref_driver.c.  The reference normally generates three small
# configuration headers with CMake; this script writes its own versions with
# the reference's default feature values (BB4D/BB6D/SC enabled, TriCub
# disabled, global aperture |x|,|y| < 1 m after every drift) into
# oracle/_ref/include instead of running the reference's build system, and
# builds the same driver twice more with other map feature flags
# (oracle/_ref/libstref_flags_{a,b}.so).
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
# config.h with the map feature flags BB4D, BB6D, SC, TRICUB (2 enabled,
# 1 skip, 0 disabled) into the include tree $1
write_config() {
mkdir -p "$1/sixtracklib/common/generated"
cat > "$1/sixtracklib/common/generated/config.h" <<EOF
#ifndef STG_REF_GENERATED_CONFIG_H
#define STG_REF_GENERATED_CONFIG_H
#define SIXTRL_TRACK_MAP_ENABLED 2
#define SIXTRL_TRACK_MAP_SKIP 1
#define SIXTRL_TRACK_MAP_DISABLED 0
#define SIXTRL_TRACK_BEAMBEAM4D $2
#define SIXTRL_TRACK_BEAMBEAM6D $3
#define SIXTRL_TRACK_SPACECHARGE $4
#define SIXTRL_TRACK_TRICUB $5
#define SIXTRL_GLOBAL_APERTURE_CHECK_ALWAYS 2
#define SIXTRL_GLOBAL_APERTURE_CHECK_CONDITIONAL 1
#define SIXTRL_GLOBAL_APERTURE_CHECK_NEVER 0
#define SIXTRL_APERTURE_CHECK_AT_DRIFT 2
#define SIXTRL_APERTURE_CHECK_MIN_DRIFT_LENGTH 0.0
#define SIXTRL_APERTURE_X_LIMIT 1.0
#define SIXTRL_APERTURE_Y_LIMIT 1.0
#endif
EOF
}
write_config "$OUT/include" 2 2 2 0
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
# Two builds with other feature flags, for the flag semantics and the
# TriCub map: (a) BB4D skip, BB6D disabled, SC skip, TriCub enabled;
# (b) BB4D disabled, BB6D skip, SC disabled, TriCub skip.
for v in "a 1 0 1 2" "b 0 1 0 1"; do
    set -- $v
    INC="$OUT/include_$1"
    write_config "$INC" "$2" "$3" "$4" "$5"
    cp "$GEN/namespace.h" "$GEN/modules.h" "$INC/sixtracklib/common/generated/"
    gcc $CFLAGS -shared -I "$INC" -I "$REF_ROOT" -I "$HERE" \
        "$HERE/ref_driver.c" -o "$OUT/libstref_flags_$1.so" -lm
done
# The reference's host-side output-buffer planning (output/output_buffer.c
# and what it calls: the elem-by-elem and beam-monitor output helpers, its
# NS(Buffer) and NS(Particles) host functions), compiled from its own eight
# source files.  -Bsymbolic keeps its st_Buffer_* calls inside this library
# when the engine's library (same C names) is loaded in the same process.
C="$REF_ROOT/sixtracklib/common"
gcc $CFLAGS -shared -Wl,-Bsymbolic -I "$OUT/include" -I "$REF_ROOT" \
    "$C/output/output_buffer.c" "$C/output/elem_by_elem_output_buffer.c" \
    "$C/output/elem_by_elem_config.c" "$C/be_monitor/output_buffer.c" \
    "$C/be_monitor/be_monitor.c" "$C/buffer/buffer.c" "$C/buffer/mem_pool.c" \
    "$C/particles/particles.c" -o "$OUT/libstref_output.so" -lm
echo "built $OUT/libstref.so"
