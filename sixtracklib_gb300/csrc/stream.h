// stream.h -- the device element stream: a CObjects lattice compiled into
// fixed-size chunks of 8-byte words that CTAs stage into shared memory with
// bulk (TMA) copies and walk as warp-uniform records.
//
// Record = header word + parameters.  Header bits: 0-7 opcode, 8-31 record
// length in words (header included), 32-63 auxiliary value (multipole order,
// slice count, flags).  One record per lattice element, in lattice order,
// so the element index is the record ordinal.  Every chunk ends with an
// OP_END record; records never straddle chunks.
#pragma once

#include <cstdint>

namespace stg {

enum Op : uint32_t {
    OP_END = 0,             // end of chunk
    OP_DRIFT = 1,           // [L]            aux bit0: global aperture check
    OP_DRIFT_EXACT = 2,     // [L]            aux bit0: global aperture check
    OP_MULTIPOLE = 3,       // [bal 0..2n+1]  aux = order n
    OP_MULTIPOLE_CURV = 4,  // [bal..., hxl, hyl, length, hxl/length, hyl/length]  aux = order n
    OP_CAVITY = 5,          // [voltage, k*frequency, deg2rad*lag]
    OP_XYSHIFT = 6,         // [-dx, -dy]
    OP_SROTATION = 7,       // [cos_z, sin_z]
    OP_LIMIT_RECT = 8,      // [min_x, max_x, min_y, max_y]
    OP_LIMIT_ELLIPSE = 9,   // [a_squ, b_squ, a_b_squ]  aux bit0: compare as floats
    OP_LIMIT_RECT_ELLIPSE = 10,  // [max_x, max_y, a_squ, b_squ, a_squ_b_squ]
    OP_DIPEDGE = 11,        // [r21, r43]
    OP_RF_MULTIPOLE = 12,   // [voltage, frequency, lag, bal..., phase...] aux = order
    OP_BB4D = 13,           // [11 BB4D data words]
    OP_BB6D = 14,           // [34 head words, n_part[N], x[N], y[N], sigma[N]]
                            // aux = N | BB6D_ROUND
    OP_SC_COASTING = 15,    // [9 SCCoasting words]
    OP_SC_QGAUSS = 16,      // [11 SCQGaussProfile words, sqrt_beta = 1 / (sqrt(2)
                            //  bunchlength_rms), sqrt_beta^2, sqrt_beta / cq,
                            //  1 / (1 - q) (0 when |1 - q| < 1e-6),
                            //  0.5 / sigma^2, 1 / (2 pi eps0 sigma),
                            //  1 / S, 1 / (2 eps0 sqrt(pi) S), sigma_y / sigma_x,
                            //  sigma_x / sigma_y, 1 / (2 sigma_x^2),
                            //  1 / (2 sigma_y^2), length N sqrt_beta / cq /
                            //  (2 pi eps0) and 1 / sigma (round; else 0)],
                            //  S = sqrt(2 |sigma_x^2 - sigma_y^2|)
                            // aux bit0 (SC_ROUND): |sigma_x - sigma_y| <
                            //  min_sigma_diff, sigma = (sigma_x + sigma_y) / 2;
                            // bit1 / bit2 (SC_ELL_X / SC_ELL_Y): elliptic with
                            //  sigma_x > sigma_y / sigma_x < sigma_y;
                            // bit3 (SC_Q1): |1 - q| < 1e-6 (Gaussian profile)
    OP_MONITOR = 17,        // [num_stores, start, skip, max_pid, min_pid, rolling,
                            //  turn_ordered, out_ptr, out_capacity]
    OP_NOP = 18,            // success, no effect (disabled beam-beam)
    OP_FAIL = 19,           // failure (map compiled out, e.g. TriCub)
    OP_FAIL_LOST = 20,      // failure and particle lost (unknown type id)
    OP_SC_INTERP = 21,      // [N, sigma_x, sigma_y, length, x_co, y_co, fallback,
                            //  min_sigma_diff, method, num_values, z0, dz,
                            //  values@, derivatives@, nwords, table address]
                            // the table (nwords words, values@ / derivatives@
                            // word offsets into it) lies in device memory
                            // outside the stream; aux bit0: interpolate (else
                            // the fallback density)
    OP_TRICUB = 22,         // [x_shift, y_shift, tau_shift, dipolar_kick_px,
                            //  dipolar_kick_py, dipolar_kick_ptau,
                            //  length / dx, length / dy, length / dz,
                            //  x0, y0, z0, 1 / dx, 1 / dy, 1 / dz,
                            //  nx - 2, ny - 2, nz - 2 (as doubles),
                            //  nx - 1, ny - 1 (cells per row / plane),
                            //  cell coefficient table address]
                            // aux bits 0-2: mirror in x, y, z.  The table (64
                            // coefficients per grid cell, x^i y^j z^k at
                            // k + 4 j + 16 i) lies in device memory outside
                            // the stream, computed there from the node table
    OP_COUNT
};

constexpr uint32_t DRIFT_APERTURE = 1u;
// TriCub aux flags: mirror the grid coordinate in x / y / z (mirror_* == 1).
constexpr uint32_t TRICUB_MIRROR_X = 1u;
constexpr uint32_t TRICUB_MIRROR_Y = 2u;
constexpr uint32_t TRICUB_MIRROR_Z = 4u;
// SC q-Gaussian aux flag: the transverse field is the round one.
constexpr uint32_t SC_ROUND = 1u;
constexpr uint32_t SC_ELL_X = 2u;
constexpr uint32_t SC_ELL_Y = 4u;
constexpr uint32_t SC_Q1 = 8u;

// BB6D aux flag: the strong beam's Sigma matrix is round and uncoupled
// (S11 = S33, S12 = S34, S22 = S44, S13 = S14 = S23 = S24 = 0) with
// threshold_singular > 0 and min_sigma_diff > 0.  Then R = S13 = 0 at every
// S, and NS(BeamBeam6D_propagate_Sigma_matrix) always takes its singular
// branch with cos theta = 1, sin theta = 0 and no theta derivative, and the
// field is the round one: the map computes only what that branch needs.
constexpr uint32_t BB6D_ROUND = 1u << 31;
constexpr uint32_t BB6D_SLICES = BB6D_ROUND - 1u;

inline uint64_t make_header(uint32_t op, uint32_t nwords, uint32_t aux)
{
    return (uint64_t)op | ((uint64_t)(nwords & 0xFFFFFFu) << 8) | ((uint64_t)aux << 32);
}

// Global aperture compare: |x| < limit  <=>  bits(|x|) < bits(limit) for a
// positive finite limit (IEEE doubles of one sign order like their bit
// patterns; NaN and inf compare false, as in the reference's float compare).
inline uint64_t aperture_bits(double limit)
{
    if (!(limit > 0.0)) return 0;  // nothing is inside a non-positive limit
    uint64_t w;
    __builtin_memcpy(&w, &limit, 8);
    return w;
}

struct StreamInfo {
    int64_t num_elements = 0;
    int32_t num_chunks = 0;
    int32_t chunk_words = 0;
    int32_t max_record_words = 0;
    int32_t num_monitors = 0;
    uint32_t op_mask = 0;  // bit per opcode present
};

}  // namespace stg
