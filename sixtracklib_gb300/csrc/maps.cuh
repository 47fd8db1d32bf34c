// maps.cuh -- element maps on the GPU, FP64, one particle per thread.
//
// Each map restates the reference map named in its comment.  The template
// flag FAST selects the arithmetic policy:
//   FAST = false: every operation rounded separately, in the reference's
//                 order (the translation unit is compiled with -fmad=false),
//                 so results are bit-identical to the reference's CPU build
//                 except where a CUDA math function (sin, exp, pow) differs
//                 from the host libm in the last bit;
//   FAST = true:  fused multiply-adds where they shorten a dependency chain
//                 (Horner kicks, drift updates, rotations); results agree
//                 with the reference to rounding level.
#pragma once

#include <cstdint>

#include "exp_table.h"
#include "stream.h"

namespace stg {

struct PState {
    double x, px, y, py, zeta, delta, psigma, rpp, rvv, chi, s;
    double beta0, q0, p0c, mass0, charge_ratio, gamma0, energy0;
    // the q-Gaussian space-charge kick's particle factors under the fast
    // policy, refreshed whenever rvv changes: chi charge_ratio (e q0)^2
    // (1 - beta0 beta) / (pc0 beta) and 1 / rvv (pc0 = p0c e, beta = beta0 rvv)
    double sc_k, inv_rvv;
    int64_t pid, at_element, at_turn, state;
    bool lazy_s;    // s is +0 at this turn's start: s is read from the lattice's s table
};

__device__ __forceinline__ double W(uint64_t w) { return __longlong_as_double((long long)w); }

// e^x for the fast arithmetic policy: P. T. P. Tang's table-driven method
// (ACM Trans. Math. Softw. 15 (1989) 144).  x = (256 m + j) ln2/256 + r with
// |r| <= ln2/512; e^x = 2^m 2^(j/256) e^r, e^r - 1 by its degree-4 Taylor
// polynomial (truncation below 4e-17 relative), 2^(j/256) from a table of
// double pairs (exp_table.h), 2^m added to the exponent field on the integer
// pipe.  Ten FP64 instructions (CUDA's exp: fifteen); within one ulp of e^x.
// |x| >= 700 (results near or beyond the normal range) and NaN take CUDA's
// exp; the test of |x| runs on the integer pipe.
__device__ __forceinline__ double exp_fast(double x)
{
    if (((uint32_t)__double2hiint(x) & 0x7FFFFFFFu) >= 0x4085E000u) return exp(x);  // |x| >= 700
    constexpr double kMagic = 6755399441055744.0;  // 1.5 * 2^52: rounds to an integer
    double const t = fma(x, kExpInvLn2N, kMagic);
    double const n = t - kMagic;
    int const N = __double2loint(t);
    double r = fma(-n, __longlong_as_double((long long)kExpL1Bits), x);
    r = fma(-n, __longlong_as_double((long long)kExpL2Bits), r);
    double q = fma(r, 1.0 / 24.0, 1.0 / 6.0);
    q = fma(q, r, 0.5);
    double const p = fma(q, r * r, r);
    int const j = N & 255;
    double const s_hi = __ldg(&kExpTable[2 * j]);
    double const s_lo = __ldg(&kExpTable[2 * j + 1]);
    double const v = s_hi + fma(s_hi, p, s_lo);
    return __hiloint2double(__double2hiint(v) + (N >> 8) * (1 << 20), __double2loint(v));
}

// 1 / d for the fast arithmetic policy: the hardware's reciprocal estimate
// (PTX rcp.approx.ftz.f64, computed from the upper 32 bits of d: about 20
// correct bits) refined by one step of the third-order iteration
// y' = y + y (e + e^2), e = 1 - d y (Householder's method of order 2 for
// f(y) = 1/y - d), which cubes the estimate's relative error to below
// 2^-57: the result is within about one ulp of 1/d.  Three FP64
// instructions.  |d| outside [2^-1000, 2^1001) -- zero, subnormals, huge
// values, inf, NaN -- takes the IEEE division; the test runs on the integer
// pipe.
__device__ __forceinline__ double rcp_fast(double d)
{
    uint32_t const e = ((uint32_t)__double2hiint(d) >> 20) & 0x7FFu;
    if (e - 23u > 2000u) return 1.0 / d;  // biased exponent outside [23, 2023]
    double y;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(d));
    double const r = fma(-d, y, 1.0);
    return fma(y, fma(r, r, r), y);
}

constexpr double kPiD = 3.1415926535897932384626433832795028841971693993751;
constexpr double kClightD = 299792458.0;
constexpr double kEps0D = 8.854187817620e-12;
constexpr double kSqrtPiD = 1.7724538509055160272981674833411451827975494561224;
constexpr double kQelemD = 1.60217662e-19;
constexpr double kCharge0SiD = 1.602176634e-19;

__device__ __forceinline__ void refresh_kick_factors(PState &p)
{
    double const pc0 = p.p0c * kCharge0SiD;
    double const beta = p.beta0 * p.rvv;
    double const inv_pc0_beta = 1.0 / (pc0 * beta);
    double const charge = kCharge0SiD * p.q0;
    p.sc_k = p.chi * p.charge_ratio * charge * charge * (1.0 - p.beta0 * beta) * inv_pc0_beta;
    p.inv_rvv = inv_pc0_beta * (pc0 * p.beta0);
}

// ------------------------------------------------------------------ energy
// NS(Particles_add_to_energy_value): particles.h:5255-5297
__device__ __forceinline__ void add_energy(PState &p, double de)
{
    double const beta0 = p.beta0;
    double const db0 = p.delta * beta0;
    double const ptau_beta0 = de / p.energy0 + sqrt(db0 * db0 + 2.0 * db0 * beta0 + 1.0) - 1.0;
    double const ptau = ptau_beta0 / beta0;
    double const psigma = ptau / beta0;
    double const delta = sqrt(ptau * ptau + 2.0 * psigma + 1.0) - 1.0;
    double const opd = delta + 1.0;
    double const rvv = opd / (1.0 + ptau_beta0);
    p.delta = delta;
    p.psigma = psigma;
    p.zeta *= rvv / p.rvv;
    p.rvv = rvv;
    p.rpp = 1.0 / opd;
    refresh_kick_factors(p);
}

// NS(Particles_update_delta_value): particles.h:5459-5496
__device__ __forceinline__ void set_delta(PState &p, double nd)
{
    double const beta0 = p.beta0;
    double const db0 = nd * beta0;
    double const ptau_beta0 = sqrt(db0 * db0 + 2.0 * db0 * beta0 + 1.0) - 1.0;
    double const opd = 1.0 + nd;
    p.delta = nd;
    p.rvv = opd / (1.0 + ptau_beta0);
    p.rpp = 1.0 / opd;
    p.psigma = ptau_beta0 / (beta0 * beta0);
    refresh_kick_factors(p);
}

// ------------------------------------------------------------------- maps
// s += L for a particle whose s is accumulated (not read from the s table).
// S_LIVE is a block-uniform property of the pass: false once every particle
// of the block reads s from the table (every turn after the first), and the
// instantiation without it has no s update at all -- a guarded add in the
// element loop would be issued (predicated off) on the FP64 pipe for every
// drift.  The add is a volatile PTX instruction so that it cannot be
// speculated out of the per-particle branch.
template <bool S_LIVE>
__device__ __forceinline__ void add_s(PState &p, double L)
{
    if constexpr (S_LIVE) {
        if (!p.lazy_s) asm volatile("add.rn.f64 %0, %0, %1;" : "+d"(p.s) : "d"(L));
    }
}

// be_drift/track.h:45-67.  FAST keeps the reference's rounding of
// 1 + (xp^2 + yp^2)/2 at the scale of 1.0 (u below): regrouping the zeta
// update as L (rvv - 1) - (L/2)(xp^2 + yp^2) is more accurate but departs
// from the reference by its own rounding noise, ~1e-16 m per drift.
// s is only accumulated when the turn did not start at s = +0 (otherwise it
// comes from the lattice's s table).
template <bool FAST, bool S_LIVE = true>
__device__ __forceinline__ void drift(PState &p, double L)
{
    double const xp = p.px * p.rpp;
    double const yp = p.py * p.rpp;
    if (FAST) {
        double const u = fma(fma(yp, yp, xp * xp), 0.5, 1.0);
        p.x = fma(xp, L, p.x);
        p.y = fma(yp, L, p.y);
        p.zeta = fma(L, p.rvv - u, p.zeta);
    } else {
        double const dzeta = p.rvv - (1.0 + (xp * xp + yp * yp) * 0.5);
        p.x += xp * L;
        p.y += yp * L;
        p.zeta += L * dzeta;
    }
    add_s<S_LIVE>(p, L);
}

// be_drift/track.h:71-97
template <bool S_LIVE = true>
__device__ __forceinline__ void drift_exact(PState &p, double L)
{
    double const opd = p.delta + 1.0;
    double const lpzi = L / sqrt(opd * opd - (p.px * p.px + p.py * p.py));
    double const dzeta = p.rvv * L - opd * lpzi;
    p.x += p.px * lpzi;
    p.y += p.py * lpzi;
    add_s<S_LIVE>(p, L);
    p.zeta += dzeta;
}

// Global aperture (be_limit/track.h:54-88) on the integer pipe:
// |x| < limit  <=>  bits(|x|) < bits(limit) for a limit >= +0; NaN and inf
// fail as in the reference's float compare.  The compare is spelled on the
// two 32-bit halves: a 64-bit mask of the sign bit is recognised as fabs()
// and costs an FP64 instruction per coordinate.
__device__ __forceinline__ bool abs_below(double v, uint64_t lim)
{
    uint32_t const hi = (uint32_t)__double2hiint(v) & 0x7FFFFFFFu;
    uint32_t const lo = (uint32_t)__double2loint(v);
    uint32_t const lhi = (uint32_t)(lim >> 32), llo = (uint32_t)lim;
    return (hi < lhi) | ((hi == lhi) & (lo < llo));
}

__device__ __forceinline__ bool inside_global(const PState &p, uint64_t xlim, uint64_t ylim)
{
    return abs_below(p.x, xlim) & abs_below(p.y, ylim);
}

// be_multipole/track.h:38-112 (bal[2k] = knl[k]/k!, bal[2k+1] = ksl[k]/k!)
// FAST: when the top-order skew coefficient is zero (a lattice without skew
// components: every multipole), the first Horner step's two products with
// it vanish and the step is two FMAs instead of four; the values are the
// four-FMA step's (a product with +-0 added to b gives b), up to the sign of
// an exact zero.  The test is on the record's bits (warp-uniform, integer
// pipe).
//
// FAST, order >= 3 and every skew coefficient zero: P(z) = sum b_k z^k has
// real coefficients, and the Goertzel / Knuth recurrence (Knuth, TAOCP
// vol. 2, 4.6.4) evaluates it with the real quadratic z^2 - 2x z + |z|^2,
// whose roots are z and its conjugate: c_n = b_n,
// c_(n-1) = b_(n-1) + 2x c_n, c_k = b_k + 2x c_(k+1) - |z|^2 c_(k+2), then
// P(z) = z c_1 - |z|^2 c_2 + b_0: 2n + 3 FP64 instructions in place of
// Horner's 4n - 2.  Its rounding matches the FMA Horner's (per-component
// deviation from the reference's Horner 1.45e-16 rms against 1.44e-16 over
// 2M random kicks of this lattice family).  The skew test ORs the record's
// odd words (warp-uniform, integer pipe): a learnable skew coefficient that
// becomes nonzero takes the Horner form again.
template <bool FAST, bool CURV>
__device__ __forceinline__ void multipole(PState &p, const uint64_t *rec, int order)
{
    const uint64_t *bal = rec + 1;
    double dpx = W(bal[2 * order]);
    double dpy = W(bal[2 * order + 1]);
    double const x = p.x, y = p.y, chi = p.chi;
    int k = order - 1;
    bool real = false;
    if (FAST && order >= 3) {
        uint64_t im = 0u;
        for (int j = 0; j <= order; ++j) im |= bal[2 * j + 1];
        real = (im << 1) == 0u;
    }
    if (FAST && real) {
        double const r = x + x;
        double const s = fma(x, x, y * y);
        double c1 = dpx;                          // c_n
        double c0 = fma(r, c1, W(bal[2 * k]));    // c_(n-1)
        for (int j = order - 2; j >= 1; --j) {
            double const cj = fma(r, c0, fma(-s, c1, W(bal[2 * j])));
            c1 = c0;
            c0 = cj;
        }
        dpx = fma(x, c0, fma(-s, c1, W(bal[0])));
        dpy = y * c0;
        k = -1;
    } else if (FAST && k >= 0 && (bal[2 * order + 1] << 1) == 0u) {
        double const nx = fma(dpx, x, W(bal[2 * k]));
        dpy = fma(dpx, y, W(bal[2 * k + 1]));
        dpx = nx;
        --k;
    }
    for (; k >= 0; --k) {
        if (FAST) {
            double const tx = fma(-dpy, y, W(bal[2 * k]));
            double const ty = fma(dpy, x, W(bal[2 * k + 1]));
            double const nx = fma(dpx, x, tx);
            dpy = fma(dpx, y, ty);
            dpx = nx;
        } else {
            double const zre = dpx * x - dpy * y;
            double const zim = dpx * y + dpy * x;
            dpx = W(bal[2 * k]) + zre;
            dpy = W(bal[2 * k + 1]) + zim;
        }
    }
    if (!CURV) {
        if (FAST) {
            p.px = fma(-chi, dpx, p.px);
            p.py = fma(chi, dpy, p.py);
        } else {
            p.px += -chi * dpx;
            p.py += chi * dpy;
        }
        return;
    }
    dpx = -chi * dpx;
    dpy = chi * dpy;
    double const hxl = W(bal[2 * order + 2]);
    double const hyl = W(bal[2 * order + 3]);
    double const length = W(bal[2 * order + 4]);
    double const hxlx = x * hxl;
    double const hyly = y * hyl;
    p.zeta += chi * (hyly - hxlx);
    dpx += hxl + hxl * p.delta;
    dpy -= hyl + hyl * p.delta;
    if (length > 0.0) {
        double const b1l = chi * W(bal[0]);
        double const a1l = chi * W(bal[1]);
        dpx -= b1l * hxlx / length;
        dpy += a1l * hyly / length;
    }
    p.px += dpx;
    p.py += dpy;
}

// be_cavity/track.h:39-67 (rec: voltage, (2 pi / c) * frequency, deg2rad * lag)
__device__ __forceinline__ void cavity(PState &p, const uint64_t *rec)
{
    double const q = p.q0 * p.charge_ratio;
    double const tau = p.zeta / (p.beta0 * p.rvv);
    double const phase = W(rec[3]) - W(rec[2]) * tau;
    double const energy = q * W(rec[1]) * sin(phase);
    add_energy(p, energy);
}

// be_srotation/track.h:38-69
template <bool FAST>
__device__ __forceinline__ void srotation(PState &p, const uint64_t *rec)
{
    double const cz = W(rec[1]), sz = W(rec[2]);
    double const x = p.x, y = p.y, px = p.px, py = p.py;
    if (FAST) {
        p.x = fma(cz, x, sz * y);
        p.y = fma(-sz, x, cz * y);
        p.px = fma(cz, px, sz * py);
        p.py = fma(-sz, px, cz * py);
    } else {
        p.x = cz * x + sz * y;
        p.y = -sz * x + cz * y;
        p.px = cz * px + sz * py;
        p.py = -sz * px + cz * py;
    }
}

// be_limit/track.h:90-111
__device__ __forceinline__ bool inside_rect(const PState &p, const uint64_t *rec)
{
    return (p.x >= W(rec[1])) && (p.x <= W(rec[2])) && (p.y >= W(rec[3])) && (p.y <= W(rec[4]));
}

// be_limit/track.h:113-137.  t <= a^2 b^2 is compared on the integer pipe
// (both sides are >= +0 or NaN; NaN fails as in the float compare) unless
// the element has negative parameters (aux bit 0).
template <bool FAST>
__device__ __forceinline__ bool inside_ellipse(const PState &p, const uint64_t *rec, uint32_t aux)
{
    double t;
    if (FAST) {
        t = fma(p.y * p.y, W(rec[1]), (p.x * p.x) * W(rec[2]));
    } else {
        t = p.x * p.x;
        t *= W(rec[2]);
        double ys = p.y * p.y;
        ys *= W(rec[1]);
        t += ys;
    }
    if (aux & 1u) return t <= W(rec[3]);
    return (uint64_t)__double_as_longlong(t) <= rec[3];
}

// be_limit/track.h:139-162
__device__ __forceinline__ bool inside_rect_ellipse(const PState &p, const uint64_t *rec)
{
    double const x = p.x, y = p.y;
    double t = x * x * W(rec[4]);
    t += y * y * W(rec[3]);
    return (x <= W(rec[1])) && (x >= -W(rec[1])) && (y <= W(rec[2])) && (y >= -W(rec[2])) &&
           (t <= W(rec[5]));
}

// be_rfmultipole/track.h:39-118
static __device__ __noinline__ PState rf_multipole(PState p, const uint64_t *rec, int order)
{
    double const voltage = W(rec[1]), frequency = W(rec[2]), lag = W(rec[3]);
    const uint64_t *bal = rec + 4;
    const uint64_t *phase = rec + 4 + 2 * order + 2;
    double const DEG2RAD = kPiD / 180.0;
    double const DEG2RAD_C = 0.0174532925199432957692369076848861271344287188854172546;
    double const k = frequency * (2.0 * kPiD) / kClightD;
    double const x = p.x, y = p.y;
    double const q = p.q0 * p.charge_ratio * 1.0;
    double const ktau = k * p.zeta / (p.beta0 * p.rvv);
    double dpx = 0.0, dpy = 0.0, dptr = 0.0, zre = 1.0, zim = 0.0;
    for (int kk = 0; kk <= order; ++kk) {
        double const pn = DEG2RAD_C * W(phase[2 * kk]) - ktau;
        double const ps = DEG2RAD * W(phase[2 * kk + 1]) - ktau;
        double const bn = W(bal[2 * kk]);
        double const bs = W(bal[2 * kk + 1]);
        double const cn = cos(pn), cs = cos(ps), sn = sin(pn), ss = sin(ps);
        dpx += cn * (bn * zre) - cs * (bs * zim);
        dpy += cs * (bs * zre) + cn * (bn * zim);
        double const zret = zre * x - zim * y;
        zim = zim * x + zre * y;
        zre = zret;
        dptr += sn * (bn * zre) - ss * (bs * zim);
    }
    double const cav_energy = q * (voltage * sin(lag * DEG2RAD_C - ktau));
    double const rfm_energy = -q * ((k * p.p0c) * dptr);
    double const chi = p.chi;
    p.px += -chi * dpx;
    p.py += chi * dpy;
    add_energy(p, cav_energy + rfm_energy);
    return p;
}

// ----------------------------------------------------- Gaussian beam fields
// Complex error function w(z): the CERN algorithm of K. Koelbig (program
// C335) as be_beamfields/faddeeva_cern.h:45-120 evaluates it -- the same
// truncated continued fraction and series (same h, nc, nu), evaluated
// without a division per term.  With U(n) the conjugate of the recursion's
// R, U(n) = 0.5 / (w0 + n U(n+1)), U(nu + 1) = 0, w0 = (y + 0.5 / h) + i x,
// is U(n) = 0.5 Q(n+1) / Q(n) for the three-term recurrence
// Q(n) = w0 Q(n+1) + (n / 2) Q(n+2), Q(nu+1) = 1, Q(nu+2) = 0; the series
// V(n) = U(n) (V(n+1) + h^(1-n)) then telescopes to
// V(1) = sum_{m=1..nc} h^(1-m) 0.5^m Q(m+1) / Q(1)
//      = 0.5 A(1) / Q(1),  A(m) = Q(m+1) + A(m+1) / (2h),  A(nc) = Q(nc+1),
// a Horner sum taken along the recurrence (two FMAs per term).  One complex
// division per call instead of two real divisions per term (|Q| stays below
// ~1e30); 0.5 / h is taken as 0.5 (3.2 q), the product h = 1 / (3.2 q) was
// formed from.  The values agree with the term-by-term evaluation to
// rounding (a few 1e-15 relative).
// The recurrence runs on a warp-uniform index: every lane of the warp steps
// through the same n, from the largest nu of the warp down, and a lane
// takes part from its own nu on (the warp issues max(nu) steps either way).
// n / 2 then comes from a table indexed by the uniform n instead of an FP64
// subtraction per step; the arithmetic of every lane is unchanged.
__constant__ double kHalfN[32] = {0.0,  0.5,  1.0,  1.5,  2.0,  2.5,  3.0,  3.5,
                                  4.0,  4.5,  5.0,  5.5,  6.0,  6.5,  7.0,  7.5,
                                  8.0,  8.5,  9.0,  9.5,  10.0, 10.5, 11.0, 11.5,
                                  12.0, 12.5, 13.0, 13.5, 14.0, 14.5, 15.0, 15.5};

// FAST: the region parameter q takes products with 1 / ylim and 1 / xlim
// (within an ulp of the quotients; nc and nu can differ only where 23 q or
// 21 q lies within an ulp of an integer), and the final complex division
// takes rcp_fast.
template <bool FAST = false>
static __device__ __noinline__ void cerrf(double in_re, double in_im, double *w_re, double *w_im)
{
    double const a_const = 1.12837916709551;
    double const xlim = 5.33, ylim = 4.29;
    double const x = fabs(in_re), y = fabs(in_im);
    double wx, wy;
    double q1r = 1.0, q1i = 0.0, q2r = 0.0, q2i = 0.0;  // Q(n+1), Q(n+2)
    if (y < ylim && x < xlim) {
        double const xr = FAST ? x * (1.0 / xlim) : x / xlim;
        double const q = (1.0 - (FAST ? y * (1.0 / ylim) : y / ylim)) * sqrt(1.0 - xr * xr);
        double const q32 = 3.2 * q;
        double const inv_2h = 0.5 * q32;  // 0.5 / h
        int const nc = 7 + (int)(23.0 * q);
        int const nu = 10 + (int)(21.0 * q);
        double const w0r = y + inv_2h, w0i = x;
        double ar = 0.0, ai = 0.0;  // A(n)
        // nu <= 31: q <= 1 for y >= 0 and x >= 0 inside the region
        int const n_top = __reduce_max_sync(__activemask(), (unsigned)nu);
        for (int n = n_top; n > 0; n--) {
            if (n <= nu) {
                double const hn = kHalfN[n];  // n / 2
                if (n <= nc) {
                    ar = fma(ar, inv_2h, q1r);
                    ai = fma(ai, inv_2h, q1i);
                }
                double const qr = fma(w0r, q1r, fma(-w0i, q1i, hn * q2r));
                double const qi = fma(w0r, q1i, fma(w0i, q1r, hn * q2i));
                q2r = q1r;
                q2i = q1i;
                q1r = qr;
                q1i = qi;
            }
        }
        // w = a_const conj(V(1)), V(1) = 0.5 A(1) / Q(1)
        double const q1sq = fma(q1r, q1r, q1i * q1i);
        double const inv = FAST ? (0.5 * a_const) * rcp_fast(q1sq) : 0.5 * a_const / q1sq;
        wx = fma(ar, q1r, ai * q1i) * inv;
        wy = fma(ar, q1i, -ai * q1r) * inv;
    } else {
        // |w0| is unbounded here: Q(n) = s^(10-n) Q'(n) with s a power of two
        // near |w0| (exact scaling), Q'(n) = (w0 / s) Q'(n+1) + (n / 2 s^2) Q'(n+2)
        int ex;
        frexp(fmax(x, y), &ex);
        double const is = ldexp(1.0, -ex);
        double const is2 = is * is;  // a power of two: every product below is exact
        double const w0r = y * is, w0i = x * is;
        for (int n = 9; n > 0; n--) {
            double const hn = (0.5 * n) * is2;
            double const qr = fma(w0r, q1r, fma(-w0i, q1i, hn * q2r));
            double const qi = fma(w0r, q1i, fma(w0i, q1r, hn * q2i));
            q2r = q1r;
            q2i = q1i;
            q1r = qr;
            q1i = qi;
        }
        // w = a_const conj(U(1)), U(1) = 0.5 Q(2) / Q(1) = 0.5 Q'(2) / (s Q'(1))
        double const q1sq = fma(q1r, q1r, q1i * q1i);
        double const inv = FAST ? (0.5 * a_const * is) * rcp_fast(q1sq) : 0.5 * a_const * is / q1sq;
        wx = fma(q2r, q1r, q2i * q1i) * inv;
        wy = fma(q2r, q1i, -q2i * q1r) * inv;
    }
    if (y == 0.) wx = exp(-x * x);
    if (in_im < 0.) {
        wx = 2.0 * exp(y * y - x * x) * cos(2.0 * x * y) - wx;
        wy = -2.0 * exp(y * y - x * x) * sin(2.0 * x * y) - wy;
        if (in_re > 0.) wy = -wy;
    } else if (in_re < 0.) {
        wy = -wy;
    }
    *w_re = wx;
    *w_im = wy;
}

// gauss_fields.h:56-208 (NS(get_Ex_Ey_Gx_Gy_gauss), centred: Delta = 0)
static __device__ __noinline__ void fields_gauss(double x, double y, double sigma_x, double sigma_y,
                                          double min_sigma_diff, int skip_gs, double *ex_p,
                                          double *ey_p, double *gx_p, double *gy_p)
{
    double ex, ey, gx = 0., gy = 0.;
    if (fabs(sigma_x - sigma_y) < min_sigma_diff) {
        double const sigma = 0.5 * (sigma_x + sigma_y);
        double const r2 = x * x + y * y;
        double t;
        if (r2 < 1e-20)
            t = sqrt(r2) / (2. * kPiD * kEps0D * sigma);
        else
            t = (1 - exp(-0.5 * r2 / (sigma * sigma))) / (2. * kPiD * kEps0D * r2);
        ex = t * x;
        ey = t * y;
        if (!skip_gs) {
            gx = 1 / (2. * (x * x + y * y)) *
                 (y * ey - x * ex +
                  1. / (2 * kPiD * kEps0D * sigma * sigma) * x * x *
                      exp(-(x * x + y * y) / (2. * sigma * sigma)));
            gy = 1. / (2 * (x * x + y * y)) *
                 (x * ex - y * ey +
                  1. / (2 * kPiD * kEps0D * sigma * sigma) * y * y *
                      exp(-(x * x + y * y) / (2. * sigma * sigma)));
        }
    } else {
        double const abx = fabs(x), aby = fabs(y);
        double S, fact, wz_re, wz_im, we_re, we_im, e;
        if (sigma_x > sigma_y) {
            S = sqrt(2. * (sigma_x * sigma_x - sigma_y * sigma_y));
            fact = 1. / (2. * kEps0D * kSqrtPiD * S);
            double const eta_re = sigma_y / sigma_x * abx;
            double const eta_im = sigma_x / sigma_y * aby;
            cerrf(abx / S, aby / S, &wz_re, &wz_im);
            cerrf(eta_re / S, eta_im / S, &we_re, &we_im);
            e = exp(-abx * abx / (2 * sigma_x * sigma_x) - aby * aby / (2 * sigma_y * sigma_y));
            ex = fact * (wz_im - we_im * e);
            ey = fact * (wz_re - we_re * e);
        } else if (sigma_x < sigma_y) {
            S = sqrt(2. * (sigma_y * sigma_y - sigma_x * sigma_x));
            fact = 1. / (2. * kEps0D * kSqrtPiD * S);
            double const eta_re = sigma_x / sigma_y * aby;
            double const eta_im = sigma_y / sigma_x * abx;
            cerrf(aby / S, abx / S, &wz_re, &wz_im);
            cerrf(eta_re / S, eta_im / S, &we_re, &we_im);
            e = exp(-aby * aby / (2 * sigma_y * sigma_y) - abx * abx / (2 * sigma_x * sigma_x));
            ey = fact * (wz_im - we_im * e);
            ex = fact * (wz_re - we_re * e);
        } else {
            ex = ey = __longlong_as_double(0x7FF0000000000000ll);  // 1/0
        }
        if (x < 0) ex = -ex;
        if (y < 0) ey = -ey;
        if (!skip_gs) {
            double const s11 = sigma_x * sigma_x, s33 = sigma_y * sigma_y;
            gx = -1. / (2 * (s11 - s33)) *
                 (x * ex + y * ey +
                  1. / (2 * kPiD * kEps0D) *
                      (sigma_y / sigma_x * exp(-x * x / (2 * s11) - y * y / (2 * s33)) - 1.));
            gy = 1. / (2 * (s11 - s33)) *
                 (x * ex + y * ey +
                  1. / (2 * kPiD * kEps0D) *
                      (sigma_x / sigma_y * exp(-x * x / (2 * s11) - y * y / (2 * s33)) - 1.));
        }
    }
    *ex_p = ex;
    *ey_p = ey;
    if (!skip_gs) {
        *gx_p = gx;
        *gy_p = gy;
    }
}

// be_beamfields/track.h:89-149
static __device__ __noinline__ PState beam_beam_4d(PState p, const uint64_t *rec)
{
    const uint64_t *d = rec + 1;
    double const charge = 1. * p.q0 * kQelemD;
    double const x = p.x - W(d[6]);
    double const y = p.y - W(d[7]);
    double const beta = p.beta0 / p.rvv;
    double const p0c = p.p0c * kQelemD;
    double ex, ey, gx, gy;
    fields_gauss(x, y, W(d[2]), W(d[3]), W(d[5]), 1, &ex, &ey, &gx, &gy);
    double const fk = p.chi * W(d[1]) * W(d[0]) * charge * (1. + beta * W(d[4])) /
                      (p0c * (beta + W(d[4])));
    p.px += (fk * ex - W(d[8]));
    p.py += (fk * ey - W(d[9]));
    return p;
}

__device__ __forceinline__ double sgn(double a) { return (double)((a >= 0) - (a < 0)); }

// be_beamfields/be_beamfields.h:2232-2385 (NS(BeamBeam6D_propagate_Sigma_matrix))
// FAST (the general branch): one reciprocal of sqrt(T) for the three
// divisions by it outside c2t, rcp_fast for 1 / (4 cos theta) and
// 1 / (4 sin theta).
template <bool FAST>
static __device__ __noinline__ void bb6d_sigma(const uint64_t *sg, double S, double thr, double *out)
{
    double const S11_0 = W(sg[0]), S12_0 = W(sg[1]), S13_0 = W(sg[2]), S14_0 = W(sg[3]),
                 S22_0 = W(sg[4]), S23_0 = W(sg[5]), S24_0 = W(sg[6]), S33_0 = W(sg[7]),
                 S34_0 = W(sg[8]), S44_0 = W(sg[9]);
    double const S11 = S11_0 + 2. * S12_0 * S + S22_0 * S * S;
    double const S33 = S33_0 + 2. * S34_0 * S + S44_0 * S * S;
    double const S13 = S13_0 + (S14_0 + S23_0) * S + S24_0 * S * S;
    double const S12 = S12_0 + S22_0 * S;
    double const S14 = S14_0 + S24_0 * S;
    double const S22 = S22_0 + 0. * S;
    double const S23 = S23_0 + S24_0 * S;
    double const S24 = S24_0 + 0. * S;
    double const S34 = S34_0 + S44_0 * S;
    double const S44 = S44_0 + 0. * S;
    double const R = S11 - S33;
    double const Wv = S11 + S33;
    double const T = R * R + 4 * S13 * S13;
    double const dS_R = 2. * (S12_0 - S34_0) + 2 * S * (S22_0 - S44_0);
    double const dS_W = 2. * (S12_0 + S34_0) + 2 * S * (S22_0 + S44_0);
    double const dS_S13 = S14_0 + S23_0 + 2 * S24_0 * S;
    double const dS_T = 2 * R * dS_R + 8. * S13 * dS_S13;
    double s11h, s33h, ct, st, ds11h, ds33h, dct, dst, c2t, dc2t;
    double const signR = sgn(R);
    if (T < thr) {
        double const a = S12 - S34;
        double const b = S22 - S44;
        double const c = S14 + S23;
        double const dd = S24;
        double sq = sqrt(a * a + c * c);
        if (sq * sq * sq < thr) {
            c2t = (fabs(dd) > thr) ? fabs(b) / sqrt(b * b + 4 * dd * dd) : 1.;
            ct = sqrt(0.5 * (1. + c2t));
            st = sgn(b) * sgn(dd) * sqrt(0.5 * (1. - c2t));
            dct = 0.;
            dst = 0.;
            s11h = 0.5 * Wv;
            s33h = 0.5 * Wv;
            ds11h = 0.5 * dS_W;
            ds33h = 0.5 * dS_W;
        } else {
            sq = sqrt(a * a + c * c);
            c2t = fabs(2. * a) / (2 * sq);
            ct = sqrt(0.5 * (1. + c2t));
            st = sgn(a) * sgn(c) * sqrt(0.5 * (1. - c2t));
            dc2t = sgn(a) * (0.5 * b / sq - a * (a * b + 2. * c * dd) / (2. * sq * sq * sq));
            dct = 1. / (4. * ct) * dc2t;
            if (fabs(st) > thr)
                dst = -1. / (4. * st) * dc2t;
            else
                dst = dd / (2. * a);
            s11h = 0.5 * Wv;
            s33h = 0.5 * Wv;
            ds11h = 0.5 * dS_W + sgn(a) * sq;
            ds33h = 0.5 * dS_W - sgn(a) * sq;
        }
    } else if (FAST) {
        // c2t keeps the IEEE square root and division: for an uncoupled
        // beam (S13 = 0) sqrt(R^2) is |R| and c2t is exactly 1, so sin theta
        // is exactly 0 -- a product with an approximate 1 / sqrt(T) would
        // leave it an ulp off 1 and sin theta ~1e-8 (or NaN above 1)
        double const sqrtT = sqrt(T);
        double const isT = rcp_fast(sqrtT);
        c2t = signR * R / sqrtT;
        ct = sqrt(0.5 * (1. + c2t));
        st = signR * sgn(S13) * sqrt(0.5 * (1. - c2t));
        s11h = 0.5 * (Wv + signR * sqrtT);
        s33h = 0.5 * (Wv - signR * sqrtT);
        dc2t = signR * (dS_R * isT - R * (0.5 * isT * isT * isT) * dS_T);
        dct = 0.25 * rcp_fast(ct) * dc2t;
        if (fabs(st) < thr)
            dst = (S14 + S23) / R;
        else
            dst = -0.25 * rcp_fast(st) * dc2t;
        ds11h = 0.5 * (dS_W + signR * 0.5 * isT * dS_T);
        ds33h = 0.5 * (dS_W - signR * 0.5 * isT * dS_T);
    } else {
        double const sqrtT = sqrt(T);
        c2t = signR * R / sqrtT;
        ct = sqrt(0.5 * (1. + c2t));
        st = signR * sgn(S13) * sqrt(0.5 * (1. - c2t));
        s11h = 0.5 * (Wv + signR * sqrtT);
        s33h = 0.5 * (Wv - signR * sqrtT);
        dc2t = signR * (dS_R / sqrtT - R / (2 * sqrtT * sqrtT * sqrtT) * dS_T);
        dct = 1. / (4. * ct) * dc2t;
        if (fabs(st) < thr)
            dst = (S14 + S23) / R;
        else
            dst = -1. / (4. * st) * dc2t;
        ds11h = 0.5 * (dS_W + signR * 0.5 / sqrtT * dS_T);
        ds33h = 0.5 * (dS_W - signR * 0.5 / sqrtT * dS_T);
    }
    out[0] = s11h;
    out[1] = s33h;
    out[2] = ct;
    out[3] = st;
    out[4] = ds11h;
    out[5] = ds33h;
    out[6] = dct;
    out[7] = dst;
}

// The round field of NS(get_Ex_Ey_Gx_Gy_gauss) with the G terms
// (gauss_fields.h:56-208) for sigma_x = sigma_y = sigma.  The reference's
// second exponential, exp(-(x^2 + y^2) / (2 sigma^2)), is the same number as
// the first, exp(-0.5 r2 / sigma^2) (both arguments are r2 / sigma^2 scaled
// by -1/2 exactly), so it is evaluated once.
// The same field and G terms from sigma^2 with two reciprocals (rcp_fast)
// and no square root (the fast arithmetic policy; within a few ulp of
// fields_round_g).
__device__ __forceinline__ void fields_round_g_fast(double x, double y, double sigma2, double *ex,
                                                    double *ey, double *gx, double *gy)
{
    constexpr double k = 1.0 / (2. * kPiD * kEps0D);
    double const inv_s2 = rcp_fast(sigma2);
    double const r2 = x * x + y * y;
    double const inv_r2 = rcp_fast(r2);
    double const e = exp_fast(-0.5 * r2 * inv_s2);
    double const t = (r2 < 1e-20) ? k * sqrt(r2 * inv_s2) : (1 - e) * k * inv_r2;
    double const exv = t * x, eyv = t * y;
    double const c = k * inv_s2;
    double const h = 0.5 * inv_r2;
    *ex = exv;
    *ey = eyv;
    *gx = h * (y * eyv - x * exv + c * x * x * e);
    *gy = h * (x * exv - y * eyv + c * y * y * e);
}

__device__ __forceinline__ void fields_round_g(double x, double y, double sigma, double *ex,
                                               double *ey, double *gx, double *gy)
{
    double const r2 = x * x + y * y;
    double const e = exp(-0.5 * r2 / (sigma * sigma));
    double const t = (r2 < 1e-20) ? sqrt(r2) / (2. * kPiD * kEps0D * sigma)
                                  : (1 - e) / (2. * kPiD * kEps0D * r2);
    double const exv = t * x, eyv = t * y;
    double const c = 1. / (2 * kPiD * kEps0D * sigma * sigma);
    double const h = 1 / (2. * r2);
    *ex = exv;
    *ey = eyv;
    *gx = h * (y * eyv - x * exv + c * x * x * e);
    *gy = h * (x * exv - y * eyv + c * y * y * e);
}

// NS(get_Ex_Ey_Gx_Gy_gauss) for the fast arithmetic policy, from the
// variances sxx = sigma_x^2 and syy = sigma_y^2 (the 6D beam-beam map has
// them before any square root): reciprocal square roots in place of the
// reference's thirteen divisions and three square roots, the Faddeeva
// function's fast form, and one exponential for the field and the G terms
// (the reference evaluates the same exponent twice).  Within a few ulp of
// fields_gauss.
static __device__ __noinline__ void fields_gauss_fast(double x, double y, double sxx, double syy,
                                                      double min_sigma_diff, double *ex_p,
                                                      double *ey_p, double *gx_p, double *gy_p)
{
    double const isx = rsqrt(sxx), isy = rsqrt(syy);
    double const sx = sxx * isx, sy = syy * isy;
    if (fabs(sx - sy) < min_sigma_diff) {
        double const sigma = 0.5 * (sx + sy);
        fields_round_g_fast(x, y, sigma * sigma, ex_p, ey_p, gx_p, gy_p);
        return;
    }
    constexpr double kFact = 1. / (2. * kEps0D * kSqrtPiD);
    constexpr double kG = 1. / (2 * kPiD * kEps0D);
    double const abx = fabs(x), aby = fabs(y);
    double const rx = abx * isx, ry = aby * isy;
    double const e = exp_fast(-0.5 * (rx * rx + ry * ry));
    double ex, ey, i2;
    double wz_re, wz_im, we_re, we_im;
    if (sxx > syy) {  // the branches on the variances: 2 (sxx - syy) keeps its sign
        double const iS = rsqrt(2. * (sxx - syy));  // 1 / S
        double const fact = kFact * iS;
        cerrf<true>(abx * iS, aby * iS, &wz_re, &wz_im);
        cerrf<true>((sy * isx) * abx * iS, (sx * isy) * aby * iS, &we_re, &we_im);
        ex = fact * (wz_im - we_im * e);
        ey = fact * (wz_re - we_re * e);
        i2 = iS * iS;  // 1 / (2 (sxx - syy))
    } else if (sxx < syy) {
        double const iS = rsqrt(2. * (syy - sxx));
        double const fact = kFact * iS;
        cerrf<true>(aby * iS, abx * iS, &wz_re, &wz_im);
        cerrf<true>((sx * isy) * aby * iS, (sy * isx) * abx * iS, &we_re, &we_im);
        ey = fact * (wz_im - we_im * e);
        ex = fact * (wz_re - we_re * e);
        i2 = -(iS * iS);
    } else {
        ex = ey = __longlong_as_double(0x7FF0000000000000ll);  // 1/0
        i2 = ex;
    }
    if (x < 0) ex = -ex;
    if (y < 0) ey = -ey;
    double const xe = x * ex + y * ey;
    *ex_p = ex;
    *ey_p = ey;
    *gx_p = -i2 * (xe + kG * ((sy * isx) * e - 1.));
    *gy_p = i2 * (xe + kG * ((sx * isy) * e - 1.));
}

// be_beamfields/track.h:342-507 with NS(BeamBeam6D_boost / inv_boost)
// (be_beamfields.h:2101-2230); rec = [hdr, 34 head words, slices...].
// ROUND: the strong beam is round and uncoupled (BB6D_ROUND): the Sigma
// propagation's singular branch reduces to Sig_11_hat = Sig_33_hat = W / 2,
// cos theta = 1, sin theta = 0, no theta derivative, and the field is the
// round one -- the same values as the general code for such a beam.
template <bool ROUND, bool FAST>
static __device__ __noinline__ PState beam_beam_6d(PState p, const uint64_t *rec, int n_slices)
{
    const uint64_t *d = rec + 1;
    const uint64_t *np_ = d + 34;
    const uint64_t *xs_ = np_ + n_slices;
    const uint64_t *ys_ = xs_ + n_slices;
    const uint64_t *ss_ = ys_ + n_slices;
    double const sphi = W(d[1]), cphi = W(d[2]), tphi = W(d[3]), salpha = W(d[4]),
                 calpha = W(d[5]);
    double const q0 = kQelemD * p.q0;
    double const P0 = p.p0c / kClightD * kQelemD;
    double x = p.x - W(d[21]) - W(d[19]);
    double px = p.px - W(d[22]);
    double y = p.y - W(d[23]) - W(d[20]);
    double py = p.py - W(d[24]);
    double sg = p.zeta - W(d[25]);
    double dl = p.delta - W(d[26]);
    // FAST: one reciprocal each for cos(phi), pz and the inverse boost's
    // determinant and one for the slices' charge factor, multiplications
    // in place of the reference's repeated divisions by them
    double const icphi = FAST ? 1. / cphi : 0.;
    {  // boost
        double const h = dl + 1. - sqrt((1. + dl) * (1. + dl) - px * px - py * py);
        double const px_st = FAST ? px * icphi - h * calpha * tphi * icphi
                                  : px / cphi - h * calpha * tphi / cphi;
        double const py_st = FAST ? py * icphi - h * salpha * tphi * icphi
                                  : py / cphi - h * salpha * tphi / cphi;
        double const dl_st = dl - px * calpha * tphi - py * salpha * tphi + h * tphi * tphi;
        double const pz_st = sqrt((1. + dl_st) * (1. + dl_st) - px_st * px_st - py_st * py_st);
        double const ipz = FAST ? 1. / pz_st : 0.;
        double const hx = FAST ? px_st * ipz : px_st / pz_st;
        double const hy = FAST ? py_st * ipz : py_st / pz_st;
        double const hs = FAST ? 1. - (dl_st + 1) * ipz : 1. - (dl_st + 1) / pz_st;
        double const L11 = 1. + hx * calpha * sphi;
        double const L12 = hx * salpha * sphi;
        double const L13 = calpha * tphi;
        double const L21 = hy * calpha * sphi;
        double const L22 = 1. + hy * salpha * sphi;
        double const L23 = salpha * tphi;
        double const L31 = hs * calpha * sphi;
        double const L32 = hs * salpha * sphi;
        double const L33 = FAST ? icphi : 1. / cphi;
        double const nx = L11 * x + L12 * y + L13 * sg;
        double const ny = L21 * x + L22 * y + L23 * sg;
        double const ns = L31 * x + L32 * y + L33 * sg;
        x = nx;
        y = ny;
        sg = ns;
        px = px_st;
        py = py_st;
        dl = dl_st;
    }
    double const thr = W(d[17]);
    double const msd = W(d[16]);
    double const kq = FAST ? W(d[0]) * q0 * (1. / (P0 * kClightD)) : 0.;
    if (ROUND && FAST) {
        // the round, uncoupled slice under the fast policy: as below, with
        // the slice's drift, Sigma terms, field and kick as FMAs, one
        // product Ksl t for both kick components, and the longitudinal kick
        // from the G terms' sum c e / 2 (the +-(y Ey - x Ex) terms of Gx
        // and Gy cancel in it)
        constexpr double k = 1.0 / (2. * kPiD * kEps0D);
        const uint64_t *sgm = d + 6;  // S11 S12 S13 S14 S22 S23 S24 S33 S34 S44
        double const S11_0 = W(sgm[0]), S12_0 = W(sgm[1]), S22_0 = W(sgm[4]);
        double const S12x2 = 2. * S12_0;
        for (int i = 0; i < n_slices; ++i) {
            double const Ksl = W(np_[i]) * kq;
            double const S = 0.5 * (sg - W(ss_[i]));
            double const xb = fma(px, S, x) - W(xs_[i]);
            double const yb = fma(py, S, y) - W(ys_[i]);
            double const s_hat = fma(fma(S22_0, S, S12x2), S, S11_0);
            double const ds_hat = 2. * fma(S, S22_0, S12_0);
            double const r2 = fma(xb, xb, yb * yb);
            double const inv_s2 = rcp_fast(s_hat);
            double const e = exp_fast(-0.5 * r2 * inv_s2);
            double const t = (r2 < 1e-20) ? k * sqrt(r2 * inv_s2) : (1 - e) * k * rcp_fast(r2);
            double const kt = Ksl * t;
            double const Fx = kt * xb, Fy = kt * yb;
            bool const on_axis = ((uint64_t)__double_as_longlong(r2) << 1) == 0u;
            double const Fz = on_axis ? __longlong_as_double(0x7FF8000000000000ll)
                                      : (0.25 * k) * Ksl * ds_hat * (e * inv_s2);
            dl = fma(0.5, fma(Fy, fma(0.5, Fy, py), Fx * fma(0.5, Fx, px)), dl + Fz);
            x = fma(-S, Fx, x);
            px = px + Fx;
            y = fma(-S, Fy, y);
            py = py + Fy;
        }
    } else {
        for (int i = 0; i < n_slices; ++i) {
            double const Ksl = FAST ? W(np_[i]) * kq : W(np_[i]) * W(d[0]) * q0 / (P0 * kClightD);
            double const S = 0.5 * (sg - W(ss_[i]));
            double const xb = x + px * S - W(xs_[i]);
            double const yb = y + py * S - W(ys_[i]);
            double Fx, Fy, Fz;
            if (ROUND) {
                // S11_0 = S33_0, S12_0 = S34_0, S22_0 = S44_0 bitwise (BB6D_ROUND),
                // so the reference's S33 is S11 to the bit, 0.5 (S11 + S33) is
                // S11, and 0.5 (2 (S12 + S34) + 2 S (S22 + S44)) is
                // 2 (S12 + S S22) exactly (scalings by powers of two)
                const uint64_t *sgm = d + 6;  // S11 S12 S13 S14 S22 S23 S24 S33 S34 S44
                double const S11_0 = W(sgm[0]), S12_0 = W(sgm[1]), S22_0 = W(sgm[4]);
                double const s_hat = S11_0 + 2. * S12_0 * S + S22_0 * S * S;
                double const ds_hat = 2. * (S12_0 + S * S22_0);
                double ex, ey, gx, gy;
                fields_round_g(xb, yb, sqrt(s_hat), &ex, &ey, &gx, &gy);
                Fx = Ksl * ex;
                Fy = Ksl * ey;
                Fz = 0.5 * (Ksl * gx * ds_hat + Ksl * gy * ds_hat);
            } else {
                double sm[8];
                bb6d_sigma<FAST>(d + 6, S, thr, sm);
                double const ct = sm[2], st = sm[3];
                double const xbh = xb * ct + yb * st;
                double const ybh = -xb * st + yb * ct;
                double const dxbh = xb * sm[6] + yb * sm[7];
                double const dybh = -xb * sm[7] + yb * sm[6];
                double ex, ey, gx = 0.0, gy = 0.0;
                if (FAST)
                    fields_gauss_fast(xbh, ybh, sm[0], sm[1], msd, &ex, &ey, &gx, &gy);
                else
                    fields_gauss(xbh, ybh, sqrt(sm[0]), sqrt(sm[1]), msd, 0, &ex, &ey, &gx, &gy);
                double const Fxh = Ksl * ex, Fyh = Ksl * ey, Gxh = Ksl * gx, Gyh = Ksl * gy;
                Fx = Fxh * ct - Fyh * st;
                Fy = Fxh * st + Fyh * ct;
                Fz = 0.5 * (Fxh * dxbh + Fyh * dybh + Gxh * sm[4] + Gyh * sm[5]);
            }
            dl = dl + Fz + 0.5 * (Fx * (px + 0.5 * Fx) + Fy * (py + 0.5 * Fy));
            x = x - S * Fx;
            px = px + Fx;
            y = y - S * Fy;
            py = py + Fy;
        }
    }
    {  // inverse boost
        double const pz = sqrt((1. + dl) * (1. + dl) - px * px - py * py);
        double const ipz = FAST ? 1. / pz : 0.;
        double const hx = FAST ? px * ipz : px / pz;
        double const hy = FAST ? py * ipz : py / pz;
        double const hs = FAST ? 1. - (dl + 1) * ipz : 1. - (dl + 1) / pz;
        double const c1 = FAST ? icphi : 1. / cphi;
        double const Det = c1 + (hx * calpha + hy * salpha - hs * sphi) * tphi;
        // Li = N / Det: FAST multiplies by one reciprocal of Det
        double const iD = FAST ? 1. / Det : 0.;
        auto over_det = [&](double num) { return FAST ? num * iD : num / Det; };
        double const Li11 = over_det(c1 + salpha * tphi * (hy - hs * salpha * sphi));
        double const Li12 = over_det(salpha * tphi * (hs * calpha * sphi - hx));
        double const Li13 =
            over_det(-tphi * (calpha - hx * salpha * salpha * sphi + hy * calpha * salpha * sphi));
        double const Li21 = over_det(calpha * tphi * (-hy + hs * salpha * sphi));
        double const Li22 = over_det(c1 + calpha * tphi * (hx - hs * calpha * sphi));
        double const Li23 =
            over_det(-tphi * (salpha - hy * calpha * calpha * sphi + hx * calpha * salpha * sphi));
        double const Li31 = over_det(-hs * calpha * sphi);
        double const Li32 = over_det(-hs * salpha * sphi);
        double const Li33 = over_det(1. + hx * calpha * sphi + hy * salpha * sphi);
        double const xi = Li11 * x + Li12 * y + Li13 * sg;
        double const yi = Li21 * x + Li22 * y + Li23 * sg;
        double const si = Li31 * x + Li32 * y + Li33 * sg;
        double const h = (dl + 1. - pz) * cphi * cphi;
        double const pxi = px * cphi + h * calpha * tphi;
        double const pyi = py * cphi + h * salpha * tphi;
        double const dli = dl + pxi * calpha * tphi + pyi * salpha * tphi - h * tphi * tphi;
        x = xi;
        y = yi;
        sg = si;
        px = pxi;
        py = pyi;
        dl = dli;
    }
    p.x = x + W(d[21]) + W(d[19]) - W(d[27]);
    p.px = px + W(d[22]) - W(d[28]);
    p.y = y + W(d[23]) + W(d[20]) - W(d[29]);
    p.py = py + W(d[24]) - W(d[30]);
    p.zeta = sg + W(d[25]) - W(d[31]);
    set_delta(p, dl + W(d[26]) - W(d[32]));
    return p;
}

// be_beamfields/track.h:154-198
static __device__ __noinline__ PState sc_coasting(PState p, const uint64_t *rec)
{
    const uint64_t *c = rec + 1;
    double const charge = kCharge0SiD * p.q0;
    double const beta0 = p.beta0;
    double const pc0 = p.p0c * kCharge0SiD;
    double fk = W(c[0]) * W(c[4]) * p.chi * p.charge_ratio * charge * charge *
                (1.0 - beta0 * beta0);
    fk /= W(c[1]) * pc0 * beta0 * p.rvv;
    double ex, ey, gx, gy;
    fields_gauss(p.x - W(c[5]), p.y - W(c[6]), W(c[2]), W(c[3]), W(c[7]), 1, &ex, &ey, &gx, &gy);
    p.px += fk * ex;
    p.py += fk * ey;
    return p;
}

// be_beamfields/track.h:203-268 with NS(Math_q_gauss) (internal/math_qgauss.h:114-175)
// FAST: the particle's 1 / (pc0 beta) gives 1 / rvv by two products, and
// a round field (aux SC_ROUND) takes its constants from the record: two
// divisions instead of four, within a few ulp of the reference's kick.
template <bool FAST>
static __device__ __noinline__ PState sc_qgauss(PState p, const uint64_t *rec, uint32_t aux)
{
    const uint64_t *c = rec + 1;
    if (FAST && (aux & SC_ROUND) && (aux & SC_Q1)) {
        // round beam, Gaussian profile: the kick is g (x, y) with
        // g = chi ... (1 - beta0 beta) / (pc0 beta) [p.sc_k]
        //     x length N sqrt_beta / cq / (2 pi eps0) [c[23]]
        //     x exp(-sqrt_beta^2 z^2) x (1 - exp(-r^2 / (2 sigma^2))) / r^2,
        // one product chain and two FMAs in place of the field vector and
        // the two kicks
        double const z = p.zeta * p.inv_rvv;
        double const ez = exp_fast(-(W(c[12]) * z * z));
        double const x = p.x - W(c[5]), y = p.y - W(c[6]);
        double const r2 = fma(x, x, y * y);
        double const fr = (r2 < 1e-20) ? sqrt(r2) * W(c[24])
                                       : (1.0 - exp_fast(-r2 * W(c[15]))) * rcp_fast(r2);
        double const g = (p.sc_k * W(c[23])) * (ez * fr);
        p.px = fma(g, x, p.px);
        p.py = fma(g, y, p.py);
        return p;
    }
    double const charge = kCharge0SiD * p.q0;
    double const beta0 = p.beta0;
    double const beta = beta0 * p.rvv;
    double const pc0 = p.p0c * kCharge0SiD;
    // FAST: the particle's factors kept since its last energy change
    double const z = FAST ? p.zeta * p.inv_rvv : p.zeta / p.rvv;
    double fk;
    if (FAST) {
        fk = p.sc_k * (W(c[4]) * W(c[0]));
    } else {
        fk = p.chi * p.charge_ratio * W(c[4]) * charge * charge * (1.0 - beta0 * beta);
        fk *= W(c[0]);
    }
    // c[11..14]: sqrt_beta = 1 / (sqrt(2) bunchlength_rms), sqrt_beta^2,
    // sqrt_beta / cq, 1 / (1 - q), computed by the lattice compiler
    double const q = W(c[8]);
    double const arg = -(W(c[12]) * z * z);
    double const omq = 1.0 - q;
    double const abs_omq = (omq >= 0.0) ? omq : -omq;
    double e;
    if (abs_omq >= 1e-6) {
        double u = 1.0 + omq * arg;
        if (u < 0.0) u = 0.0;
        e = pow(u, W(c[14]));
    } else {
        e = FAST ? exp_fast(arg) : exp(arg);
    }
    fk *= W(c[13]) * e;
    double ex, ey, gx, gy;
    if (FAST) {
        if (aux & SC_ROUND) {
            double const x = p.x - W(c[5]), y = p.y - W(c[6]);
            double const r2 = x * x + y * y;
            double const t = (r2 < 1e-20) ? sqrt(r2) * W(c[16])
                                          : (1.0 - exp_fast(-r2 * W(c[15]))) *
                                                (1.0 / (2. * kPiD * kEps0D)) * rcp_fast(r2);
            ex = t * x;
            ey = t * y;
        } else if (aux & (SC_ELL_X | SC_ELL_Y)) {
            // the elliptic field with its element constants from the record
            double const x = p.x - W(c[5]), y = p.y - W(c[6]);
            double const abx = fabs(x), aby = fabs(y);
            double const is = W(c[17]), fact = W(c[18]);
            double const e = exp_fast(-(abx * abx * W(c[21])) - aby * aby * W(c[22]));
            double wz_re, wz_im, we_re, we_im;
            if (aux & SC_ELL_X) {
                cerrf<true>(abx * is, aby * is, &wz_re, &wz_im);
                cerrf<true>(W(c[19]) * abx * is, W(c[20]) * aby * is, &we_re, &we_im);
                ex = fact * (wz_im - we_im * e);
                ey = fact * (wz_re - we_re * e);
            } else {
                cerrf<true>(aby * is, abx * is, &wz_re, &wz_im);
                cerrf<true>(W(c[20]) * aby * is, W(c[19]) * abx * is, &we_re, &we_im);
                ey = fact * (wz_im - we_im * e);
                ex = fact * (wz_re - we_re * e);
            }
            if (x < 0) ex = -ex;
            if (y < 0) ey = -ey;
        } else {
            fields_gauss(p.x - W(c[5]), p.y - W(c[6]), W(c[2]), W(c[3]), W(c[7]), 1, &ex, &ey,
                         &gx, &gy);
        }
    } else {
        fk /= pc0 * beta;
        fields_gauss(p.x - W(c[5]), p.y - W(c[6]), W(c[2]), W(c[3]), W(c[7]), 1, &ex, &ey, &gx,
                     &gy);
    }
    p.px += fk * ex;
    p.py += fk * ey;
    return p;
}

// NS(LineDensityProfileData_interpolate_value), be_beamfields.h:3385-3408,
// with NS(Math_interpol_y_equ), internal/math_interpol.h:649-665 (linear)
// and :789-816 (cubic).  c: the record's parameters; the tables are one
// window of memory holding both arrays (values at word c[12], derivatives
// at c[13], c[14] words), copied in at compile time; a read outside the
// window gives 0.
__device__ __forceinline__ double ldp_word(const uint64_t *c, uint64_t off, int64_t i)
{
    uint64_t const k = off + (uint64_t)i;
    const double *table = reinterpret_cast<const double *>(c[15]);
    return (i >= 0 && k < c[14]) ? __ldg(table + k) : 0.0;
}

__device__ __forceinline__ double ldp_interpolate(const uint64_t *c, double z)
{
    uint64_t const method = c[8];
    int64_t const nv = (int64_t)c[9];
    double const z0 = W(c[10]), dz = W(c[11]);
    double result = 0.0;
    if ((z <= z0 + dz * (double)nv) && (z >= z0)) {
        int64_t const idx = (int64_t)((z - z0) / dz);
        if (method == 0) {
            result = ldp_word(c, c[12], idx) + (z - (z0 + dz * (double)idx)) * ldp_word(c, c[13], idx);
        } else if (method == 1) {
            double const t2 = (z0 + dz * (double)(idx + 1) - z) / dz;
            double const t1 = (z - (z0 + dz * (double)idx)) / dz;
            double y = ldp_word(c, c[12], idx + 1) * t1 + ldp_word(c, c[12], idx) * t2;
            y -= ldp_word(c, c[13], idx) * dz * dz * (t2 - t2 * t2 * t2) / 6.0;
            y -= ldp_word(c, c[13], idx + 1) * dz * dz * (t1 - t1 * t1 * t1) / 6.0;
            result = y;
        }
    }
    return result;
}

// be_beamfields/track.h:273-337
static __device__ __noinline__ PState sc_interpolated(PState p, const uint64_t *rec, uint32_t aux)
{
    const uint64_t *c = rec + 1;
    double const charge = kCharge0SiD * p.q0;
    double const beta0 = p.beta0;
    double const beta = beta0 * p.rvv;
    double const pc0 = p.p0c * kCharge0SiD;
    double fk = p.chi * p.charge_ratio * W(c[3]) * W(c[0]) * charge * charge *
                (1.0 - beta0 * beta);
    if (aux & 1u)
        fk *= ldp_interpolate(c, p.zeta);
    else
        fk *= W(c[6]);
    fk /= (pc0 * beta);
    double ex, ey, gx, gy;
    fields_gauss(p.x - W(c[4]), p.y - W(c[5]), W(c[1]), W(c[2]), W(c[7]), 1, &ex, &ey, &gx, &gy);
    p.px += fk * ex;
    p.py += fk * ey;
    return p;
}

// be_tricub/track.h:51-224: the kick of a tricubic interpolant of a
// potential on a regular grid.  c: the record's parameters (stream.h
// OP_TRICUB); the cell's 64 polynomial coefficients come from the table the
// uploader computed (tricub.cu) with the reference's arithmetic, so they
// equal the ones NS(tricub_construct_coefs) forms per particle.  The
// reference reads outside its table for a particle outside the grid (only a
// debug assertion guards it); here such a particle is lost and the map fails
// (state 0 on return).
//   exact: the three derivative sums term by term in the reference's order
//          (i, then j, then k; each term ((c x^i) y^j) z^k times the power);
//   fast:  the sums as nested Horner forms over z, y and x with FMAs, the
//          derivative weights (2u, 3u^2) taken into the powers once.
template <bool FAST>
static __device__ __noinline__ PState tricub(PState p, const uint64_t *rec, uint32_t aux)
{
    const uint64_t *c = rec + 1;
    double const z = p.zeta / (p.beta0 * p.rvv);
    double const fx = ((p.x - W(c[0])) - W(c[9])) * W(c[12]);
    double const fy = ((p.y - W(c[1])) - W(c[10])) * W(c[13]);
    double const fz = ((z - W(c[2])) - W(c[11])) * W(c[14]);
    double const sign_x = ((aux & TRICUB_MIRROR_X) && fx < 0.0) ? -1. : 1.;
    double const sign_y = ((aux & TRICUB_MIRROR_Y) && fy < 0.0) ? -1. : 1.;
    double const sign_z = ((aux & TRICUB_MIRROR_Z) && fz < 0.0) ? -1. : 1.;
    double const sfx = sign_x * fx, sfy = sign_y * fy, sfz = sign_z * fz;
    double const ixf = floor(sfx), iyf = floor(sfy), izf = floor(sfz);
    // inside the grid: 0 <= i <= n - 2 in every coordinate (NaN fails)
    if (!(ixf >= 0.0 && ixf <= W(c[15]) && iyf >= 0.0 && iyf <= W(c[16]) && izf >= 0.0 &&
          izf <= W(c[17]))) {
        p.state = 0;
        return p;
    }
    int64_t const ix = (int64_t)ixf, iy = (int64_t)iyf, iz = (int64_t)izf;
    double const xn = sfx - ixf, yn = sfy - iyf, zn = sfz - izf;
    const double *cf = reinterpret_cast<const double *>(c[20]) +
                       64 * (ix + (int64_t)c[18] * (iy + (int64_t)c[19] * iz));
    double kpx, kpy, kpt;
    if (FAST) {
        // derivative weights taken into the powers once: d/du of
        // c0 + c1 u + c2 u^2 + c3 u^3 is c1 + c2 (2u) + c3 (3u^2)
        double const z2 = 2.0 * zn, z3 = 3.0 * (zn * zn);
        double const y2 = 2.0 * yn, y3 = 3.0 * (yn * yn);
        double const x2 = 2.0 * xn, x3 = 3.0 * (xn * xn);
        double dfy = 0.0, dfz = 0.0, R1 = 0.0, R2 = 0.0, R3 = 0.0;
#pragma unroll
        for (int i = 3; i >= 0; --i) {
            double P[4], Q[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                double2 const a = __ldg(reinterpret_cast<const double2 *>(cf + 4 * j + 16 * i));
                double2 const b = __ldg(reinterpret_cast<const double2 *>(cf + 4 * j + 16 * i + 2));
                // P = sum_k c_ijk z^k, Q = dP/dz
                P[j] = fma(fma(fma(b.y, zn, b.x), zn, a.y), zn, a.x);
                Q[j] = fma(b.y, z3, fma(b.x, z2, a.y));
            }
            double const R = fma(fma(fma(P[3], yn, P[2]), yn, P[1]), yn, P[0]);  // sum_j P y^j
            double const S = fma(P[3], y3, fma(P[2], y2, P[1]));                 // d/dy
            double const T = fma(fma(fma(Q[3], yn, Q[2]), yn, Q[1]), yn, Q[0]);  // d/dz
            if (i == 3) R3 = R;
            if (i == 2) R2 = R;
            if (i == 1) R1 = R;
            dfy = fma(dfy, xn, S);
            dfz = fma(dfz, xn, T);
        }
        kpx = fma(R3, x3, fma(R2, x2, R1));
        kpy = dfy;
        kpt = dfz;
    } else {
        double const x2 = xn * xn, y2 = yn * yn, z2 = zn * zn;
        double const xp[4] = {1., xn, x2, x2 * xn};
        double const yp[4] = {1., yn, y2, y2 * yn};
        double const zp[4] = {1., zn, z2, z2 * zn};
        kpx = 0.;
#pragma unroll
        for (int i = 1; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j)
#pragma unroll
                for (int k = 0; k < 4; ++k)
                    kpx += (double)i * (((__ldg(cf + k + 4 * j + 16 * i) * xp[i - 1]) * yp[j]) * zp[k]);
        kpy = 0.;
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 1; j < 4; ++j)
#pragma unroll
                for (int k = 0; k < 4; ++k)
                    kpy += (double)j * (((__ldg(cf + k + 4 * j + 16 * i) * xp[i]) * yp[j - 1]) * zp[k]);
        kpt = 0.;
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j)
#pragma unroll
                for (int k = 1; k < 4; ++k)
                    kpt += (double)k * (((__ldg(cf + k + 4 * j + 16 * i) * xp[i]) * yp[j]) * zp[k - 1]);
    }
    kpx *= W(c[6]);
    kpx *= -sign_x;
    kpx -= W(c[3]);
    kpy *= W(c[7]);
    kpy *= -sign_y;
    kpy -= W(c[4]);
    kpt *= W(c[8]);
    kpt *= -sign_z;
    kpt -= W(c[5]);
    double const q = p.q0 * p.charge_ratio;
    double const energy_kick = q * (p.p0c * kpt);
    p.px += kpx;
    p.py += kpy;
    add_energy(p, energy_kick);
    return p;
}

}  // namespace stg
