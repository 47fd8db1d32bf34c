// adjoint.cu -- reverse-mode derivative of until-turn tracking.
//
// For a loss L on the particles' final coordinates u = (x, px, y, py, zeta,
// delta), the adjoint lambda = dL/du is carried backwards through the
// lattice: lambda_in = J^T lambda_out for each map, J being the map's
// Jacobian with rpp and rvv taken as the functions of delta that
// NS(Particles_update_delta_value) defines (particles.h:5459-5496).
// Derivatives with respect to element parameters (multipole coefficients
// bal[k], cavity voltage) are accumulated over particles and turns.
//
// Every differentiable map here is explicitly invertible (drifts and
// rotations trivially, thin kicks because they leave x and y unchanged, the
// cavity because it preserves tau = zeta / (beta0 rvv), the 6D beam-beam
// slice by slice).  So the reverse
// sweep needs no tape: each thread holds one particle's state and adjoint in
// registers and, for each element, last to first, restores the element's
// input from its output and applies the transposed Jacobian at that input.
// One launch reverses a range of turns [turn_begin, turn_end) from the
// states stored at both ends: a particle starts from its state at
// turn_end, or, if it was lost inside the range, from the element where it
// stopped (its at_turn / at_element).  The reconstruction error grows by
// rounding each element; callers bound it by re-anchoring at stored turn
// boundaries (every turn when the caller recomputes the per-turn states,
// every checkpoint otherwise).
//
// All lanes of a warp walk the same element at the same time, so parameter
// contributions are reduced with warp shuffles, summed per CTA in shared
// memory and added to the global gradient once per CTA and launch.
//
// Apertures contribute no derivative (a loss is a discontinuity).  Lattices
// with elements that have no adjoint (the TriCub map, disabled maps and
// unknown type ids) are refused before launch.
#include <cuda_runtime.h>

#include <string>

#include "common.h"
#include "device_guard.h"
#include "kernel_api.h"
#include "lattice_view.h"
#include "dual.cuh"
#include "maps.cuh"

namespace stg {

namespace {

constexpr int kAdjThreads = 128;
// 3 CTAs per SM: at most 168 registers a thread, which the walk over the
// ordinary maps needs without spilling; the out-of-line beam-beam and
// space-charge reverses spill into the stack instead of lowering the
// occupancy of every lattice's sweep
constexpr int kAdjBlocksPerSm = 3;

// Parameter sums: per-thread columns in shared memory while they fit
// (no reduction on the FP64 pipe until the end of the launch), else per-CTA
// slots fed by warp reductions, else global atomics.
constexpr int kMaxColumnSlots = 96;   // 96 x 128 threads x 8 B = 96 KiB
constexpr int kMaxSmemSlots = 4096;   // 32 KiB
enum AccMode : int32_t { ACC_GLOBAL = 0, ACC_CTA = 1, ACC_COLUMNS = 2 };

struct AdjParams {
    const uint64_t *stream;
    const int64_t *elem_offset;
    int64_t num_elements;
    const uint64_t *start;   // 21 x n: states at turn_begin
    const uint64_t *end;     // 21 x n: states at turn_end
    int64_t n;
    int64_t turn_begin, turn_end;
    const int64_t *idx;      // particles alive at turn_begin with work before turn_end
    const int64_t *count;
    double *lam;             // 6 x n (x px y py zeta delta): in end of turn, out start
    const int32_t *pbeg;     // num_elements + 1 offsets into the parameter list (or null)
    const int32_t *pkind;    // bal index (>= 0) or -1 for a cavity voltage
    const int32_t *pid;      // gradient slot of the entry
    double *grad;            // dL/d(bal or voltage) per gradient slot
    int32_t slots;           // number of gradient slots
    int32_t acc;             // AccMode
};

struct Lam {
    double x, px, y, py, z, d;
};

struct RState {
    double x, px, y, py, zeta, delta, rpp, rvv;
    // functions of delta (and of lambda_zeta), constant between cavities
    double drvv;    // d rvv / d delta
    double drpp;    // d rpp / d delta = -rpp^2
    double rvvm1;   // rvv - 1
    double hr2;     // rpp^2 / 2
    double lzr;     // lambda_zeta * rpp
    double lzdrvv;  // lambda_zeta * d rvv / d delta
    double beta0, chi, q, energy0, p0c, q0, cr;  // q = q0 * charge_ratio (cr)
};

// Q(delta) = sqrt(delta^2 b0^2 + 2 delta b0^2 + 1) = 1 + ptau * beta0
__device__ __forceinline__ double q_of_delta(double delta, double beta0)
{
    double const db0 = delta * beta0;
    return sqrt(db0 * db0 + 2.0 * db0 * beta0 + 1.0);
}

__device__ __forceinline__ double warp_sum(double v)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
    return v;
}

__device__ __forceinline__ double drvv_of(double delta, double beta0)
{
    double const Q = q_of_delta(delta, beta0);
    return (1.0 - beta0 * beta0) / (Q * Q * Q);
}

// Refresh the cached terms after delta or lambda_zeta changed (start of the
// walk, cavities); drifts and kicks leave both unchanged.
__device__ __forceinline__ void set_delta_terms(RState &s, double lz)
{
    s.drvv = drvv_of(s.delta, s.beta0);
    s.drpp = -s.rpp * s.rpp;
    s.rvvm1 = s.rvv - 1.0;
    s.hr2 = 0.5 * s.rpp * s.rpp;
    s.lzr = lz * s.rpp;
    s.lzdrvv = lz * s.drvv;
}

extern __shared__ double s_grad[];

// `on` lanes contribute g; all lanes of the warp call this together.
__device__ __forceinline__ void add_grad(const AdjParams &a, int32_t j, double g, bool on)
{
    if (a.acc == ACC_COLUMNS) {
        if (on) s_grad[a.pid[j] * kAdjThreads + threadIdx.x] += g;
        return;
    }
    g = warp_sum(on ? g : 0.0);
    if ((threadIdx.x & 31) == 0 && g != 0.0) {
        if (a.acc == ACC_CTA)
            atomicAdd(&s_grad[a.pid[j]], g);
        else
            atomicAdd(&a.grad[a.pid[j]], g);
    }
}

// P(z) = sum_k (bal[2k] + i bal[2k+1]) z^k and P'(z), z = x + i y, by Horner.
__device__ __forceinline__ void horner2(const uint64_t *bal, int n, double x, double y,
                                        double &pr, double &pi, double &dr, double &di)
{
    pr = W(bal[2 * n]);
    pi = W(bal[2 * n + 1]);
    dr = 0.0;
    di = 0.0;
    // a zero top-order skew coefficient (a lattice without skew components)
    // drops the products with it from the first step of P and of P' (the
    // forward map does the same; equal values up to the sign of an exact zero)
    bool const real_top = (bal[2 * n + 1] << 1) == 0u;
    int k = n - 2;
    if (n > 0) {  // first step: P' = a_n, P = a_n z + a_(n-1)
        dr = pr;
        di = pi;
        double npr, npi;
        if (real_top) {
            npr = fma(pr, x, W(bal[2 * n - 2]));
            npi = fma(pr, y, W(bal[2 * n - 1]));
        } else {
            npr = fma(pr, x, fma(-pi, y, W(bal[2 * n - 2])));
            npi = fma(pr, y, fma(pi, x, W(bal[2 * n - 1])));
        }
        pr = npr;
        pi = npi;
        if (real_top && k >= 0) {  // P' = a_n z + P with di = 0
            double const ndr = fma(dr, x, pr);
            double const ndi = fma(dr, y, pi);
            double const npr2 = fma(pr, x, fma(-pi, y, W(bal[2 * k])));
            double const npi2 = fma(pr, y, fma(pi, x, W(bal[2 * k + 1])));
            dr = ndr;
            di = ndi;
            pr = npr2;
            pi = npi2;
            --k;
        }
    }
    for (; k >= 0; --k) {
        double const ndr = fma(dr, x, fma(-di, y, pr));
        double const ndi = fma(dr, y, fma(di, x, pi));
        double const npr = fma(pr, x, fma(-pi, y, W(bal[2 * k])));
        double const npi = fma(pr, y, fma(pi, x, W(bal[2 * k + 1])));
        dr = ndr;
        di = ndi;
        pr = npr;
        pi = npi;
    }
}

__device__ __forceinline__ void refresh_lz(RState &s, const Lam &l)
{
    s.lzr = l.z * s.rpp;
    s.lzdrvv = l.z * s.drvv;
}

// Reverse of NS(Particles_add_to_energy_value) (particles.h:5255-5297) for
// an energy change dE (in units of energy0) that the caller knows from the
// map's output: restores delta, rvv, rpp and zeta (zeta *= rvv_new / rvv_old
// is undone), applies the transposed Jacobian of the direct dependencies
// and returns lambda_P, the adjoint of P = dE + Q(delta) - 1, from which the
// caller adds the terms of dE's own dependencies.  Call refresh_lz after
// the last change to lambda_zeta.
__device__ __forceinline__ double reverse_add_energy(RState &s, Lam &l, double dEn)
{
    double const beta0 = s.beta0, b2 = beta0 * beta0;
    double const zeta_o = s.zeta, rvv_o = s.rvv, delta_o = s.delta;
    double const Qo = q_of_delta(delta_o, beta0);
    double const P = b2 * delta_o * (delta_o + 2.0) / (Qo + 1.0);  // Qo - 1
    double const opdn = 1.0 + delta_o;
    // input: Q_in - 1 = P - dE / E0
    double const qm1 = P - dEn;
    double const Qi = 1.0 + qm1;
    double const r = qm1 * (qm1 + 2.0) / b2;  // (1 + delta_in)^2 - 1
    double const opd = sqrt(r + 1.0);
    double const rvv = opd / Qi;
    double const zeta = zeta_o * rvv / rvv_o;
    s.delta = r / (opd + 1.0);
    s.rvv = rvv;
    s.rpp = 1.0 / opd;
    s.zeta = zeta;
    double const drvv = (1.0 - b2) / (Qi * Qi * Qi);
    s.drvv = drvv;
    s.drpp = -s.rpp * s.rpp;
    s.rvvm1 = rvv - 1.0;
    s.hr2 = 0.5 * s.rpp * s.rpp;
    double const dopd_dP = (1.0 + P) / (b2 * opdn);
    double const drvvn_dP = dopd_dP / (1.0 + P) - opdn / ((1.0 + P) * (1.0 + P));
    double const lP = l.d * dopd_dP + l.z * (zeta / rvv) * drvvn_dP;
    double const lz = l.z * (rvv_o / rvv);
    l.d = -l.z * (zeta * rvv_o / (rvv * rvv)) * drvv + lP * (b2 * opd / Qi);
    l.z = lz;
    return lP;
}

// Adjoint of tau = zeta / (beta0 rvv(delta)) at the (restored) input.
__device__ __forceinline__ void add_tau_adjoint(const RState &s, Lam &l, double ltau)
{
    double const br = s.beta0 * s.rvv;
    l.z += ltau / br;
    l.d -= ltau * s.zeta / (br * s.rvv) * s.drvv;
}

// The Gaussian field of NS(get_Ex_Ey_Gx_Gy_gauss) without the G terms
// (be_beamfields/gauss_fields.h:56-208), as the forward kernel computes it,
// and its Jacobian d(Ex, Ey)/d(x, y).  Elliptic beams: d w / d z = -2 z w +
// 2 i / sqrt(pi) evaluated with the same w(z) (CERN algorithm), so the
// Jacobian is that of the exact Faddeeva function at the approximated w.
struct FieldJ {
    double ex, ey, exx, exy, eyx, eyy;
};

__device__ __noinline__ FieldJ field_jacobian(double x, double y, double sigma_x, double sigma_y,
                                              double min_sigma_diff)
{
    FieldJ f{};
    if (fabs(sigma_x - sigma_y) < min_sigma_diff) {
        double const sigma = 0.5 * (sigma_x + sigma_y);
        double const r2 = x * x + y * y;
        double t, dt;  // dt = d t / d r2
        if (r2 < 1e-20) {
            t = sqrt(r2) / (2. * kPiD * kEps0D * sigma);
            dt = (r2 > 0.0) ? t / (2.0 * r2) : 0.0;
        } else {
            double const e = exp(-0.5 * r2 / (sigma * sigma));
            t = (1 - e) / (2. * kPiD * kEps0D * r2);
            dt = (e / (2. * kPiD * kEps0D * 2.0 * sigma * sigma) - t) / r2;
        }
        f.ex = t * x;
        f.ey = t * y;
        f.exx = t + 2.0 * x * x * dt;
        f.exy = 2.0 * x * y * dt;
        f.eyx = f.exy;
        f.eyy = t + 2.0 * y * y * dt;
        return f;
    }
    double const abx = fabs(x), aby = fabs(y);
    double const sgn_xy = ((x < 0) != (y < 0)) ? -1.0 : 1.0;
    double const two_isqpi = 2.0 / kSqrtPiD;
    // first quadrant: u along the wider axis, v along the other
    bool const xwide = sigma_x > sigma_y;
    if (!(sigma_x > sigma_y) && !(sigma_x < sigma_y)) return f;  // the reference's 1/0
    double const su = xwide ? sigma_x : sigma_y, sv = xwide ? sigma_y : sigma_x;
    double const au = xwide ? abx : aby, av = xwide ? aby : abx;
    double const S = sqrt(2. * (su * su - sv * sv));
    double const fact = 1. / (2. * kEps0D * kSqrtPiD * S);
    double const eta_re = sv / su * au, eta_im = su / sv * av;
    double z1r = au / S, z1i = av / S, z2r = eta_re / S, z2i = eta_im / S;
    double w1r, w1i, w2r, w2i;
    cerrf(z1r, z1i, &w1r, &w1i);
    cerrf(z2r, z2i, &w2r, &w2i);
    double const e = exp(-au * au / (2 * su * su) - av * av / (2 * sv * sv));
    // fields along (v, u): Fv = fact (Im w1 - Im w2 e), Fu = fact (Re w1 - Re w2 e)
    double const fv = fact * (w1i - w2i * e);
    double const fu = fact * (w1r - w2r * e);
    // w'(z) = -2 z w + 2 i / sqrt(pi)
    double const d1r = -2.0 * (z1r * w1r - z1i * w1i), d1i = -2.0 * (z1r * w1i + z1i * w1r) + two_isqpi;
    double const d2r = -2.0 * (z2r * w2r - z2i * w2i), d2i = -2.0 * (z2r * w2i + z2i * w2r) + two_isqpi;
    // d/du: w1 -> d1 / S, w2 -> d2 (sv / su) / S, e -> -au / su^2 e
    // d/dv: w1 -> i d1 / S, w2 -> i d2 (su / sv) / S, e -> -av / sv^2 e
    double const cu2 = sv / su / S, cv2 = su / sv / S;
    double const eu = -au / (su * su) * e, ev = -av / (sv * sv) * e;
    double const fv_u = fact * (d1i / S - (d2i * cu2 * e + w2i * eu));
    double const fv_v = fact * (d1r / S - (d2r * cv2 * e + w2i * ev));
    double const fu_u = fact * (d1r / S - (d2r * cu2 * e + w2r * eu));
    double const fu_v = fact * (-d1i / S - (-d2i * cv2 * e + w2r * ev));
    // map back: the wide axis carries Fv (Ex for sigma_x > sigma_y)
    double exq, eyq, ex_x, ex_y, ey_x, ey_y;
    if (xwide) {  // u = x, v = y: Ex = Fv, Ey = Fu
        exq = fv;
        eyq = fu;
        ex_x = fv_u;
        ex_y = fv_v;
        ey_x = fu_u;
        ey_y = fu_v;
    } else {      // u = y, v = x: Ey = Fv, Ex = Fu
        eyq = fv;
        exq = fu;
        ey_y = fv_u;
        ey_x = fv_v;
        ex_y = fu_u;
        ex_x = fu_v;
    }
    f.ex = (x < 0) ? -exq : exq;
    f.ey = (y < 0) ? -eyq : eyq;
    f.exx = ex_x;
    f.eyy = ey_y;
    f.exy = sgn_xy * ex_y;
    f.eyx = sgn_xy * ey_x;
    return f;
}

// A thin transverse kick px += K E_x(x - x0, y - y0) - cx, py += K E_y - cy
// with K depending on delta and zeta: restore px, py and apply the
// transposed Jacobian.
__device__ __forceinline__ void reverse_field_kick(RState &s, Lam &l, const FieldJ &f, double K,
                                                   double dK_ddelta, double dK_dzeta, double cx,
                                                   double cy)
{
    s.px -= K * f.ex - cx;
    s.py -= K * f.ey - cy;
    double const lpx = l.px, lpy = l.py;
    l.x += K * (lpx * f.exx + lpy * f.eyx);
    l.y += K * (lpx * f.exy + lpy * f.eyy);
    double const le = lpx * f.ex + lpy * f.ey;
    l.d += le * dK_ddelta;
    l.z += le * dK_dzeta;
}

// q-Gaussian line density and its derivative (internal/math_qgauss.h:114-175)
__device__ __forceinline__ double q_gauss_d(double z, double q, double sqrt_beta, double cq,
                                            double *dq_dz)
{
    double const arg = -(sqrt_beta * sqrt_beta * z * z);
    double const darg = -2.0 * sqrt_beta * sqrt_beta * z;
    double const omq = 1.0 - q;
    double const abs_omq = (omq >= 0.0) ? omq : -omq;
    double e, de;
    if (abs_omq >= 1e-6) {
        double u = 1.0 + omq * arg;
        if (u < 0.0) u = 0.0;
        e = pow(u, 1.0 / omq);
        de = (u > 0.0) ? e / u * darg : 0.0;
    } else {
        e = exp(arg);
        de = e * darg;
    }
    *dq_dz = (sqrt_beta / cq) * de;
    return (sqrt_beta / cq) * e;
}

// d lambda / d z of the tabulated line density (see ldp_interpolate)
__device__ __forceinline__ double ldp_slope(const uint64_t *c, double z)
{
    uint64_t const method = c[8];
    int64_t const nv = (int64_t)c[9];
    double const z0 = W(c[10]), dz = W(c[11]);
    if (!((z <= z0 + dz * (double)nv) && (z >= z0))) return 0.0;
    int64_t const idx = (int64_t)((z - z0) / dz);
    if (method == 0) return ldp_word(c, c[13], idx);
    if (method == 1) {
        double const t2 = (z0 + dz * (double)(idx + 1) - z) / dz;
        double const t1 = (z - (z0 + dz * (double)idx)) / dz;
        return (ldp_word(c, c[12], idx + 1) - ldp_word(c, c[12], idx)) / dz +
               ldp_word(c, c[13], idx) * dz * (1.0 - 3.0 * t2 * t2) / 6.0 -
               ldp_word(c, c[13], idx + 1) * dz * (1.0 - 3.0 * t1 * t1) / 6.0;
    }
    return 0.0;
}

// be_rfmultipole/track.h:39-118: kicks of px, py and an energy change, all
// functions of x, y and tau = zeta / (beta0 rvv), which the map preserves.
__device__ __forceinline__ void reverse_rf_multipole_impl(RState &s, Lam &l, const uint64_t *rec,
                                                          int order)
{
    double const voltage = W(rec[1]), frequency = W(rec[2]), lag = W(rec[3]);
    const uint64_t *bal = rec + 4;
    const uint64_t *phase = rec + 4 + 2 * order + 2;
    double const DEG2RAD = kPiD / 180.0;
    double const DEG2RAD_C = 0.0174532925199432957692369076848861271344287188854172546;
    double const k = frequency * (2.0 * kPiD) / kClightD;
    double const x = s.x, y = s.y, chi = s.chi;
    double const ktau = k * s.zeta / (s.beta0 * s.rvv);
    double dpx = 0, dpy = 0, dptr = 0, zre = 1.0, zim = 0.0, pre = 0.0, pim = 0.0;
    double dpx_x = 0, dpx_y = 0, dpx_t = 0, dpy_x = 0, dpy_y = 0, dpy_t = 0;
    double dptr_x = 0, dptr_y = 0, dptr_t = 0;
    for (int kk = 0; kk <= order; ++kk) {
        double sn, cn, ss, cs;
        sincos(DEG2RAD_C * W(phase[2 * kk]) - ktau, &sn, &cn);
        sincos(DEG2RAD * W(phase[2 * kk + 1]) - ktau, &ss, &cs);
        double const bn = W(bal[2 * kk]), bs = W(bal[2 * kk + 1]);
        // d z^kk / dx = kk z^(kk-1), d z^kk / dy = i kk z^(kk-1)
        double const ar = kk * pre, ai = kk * pim;
        dpx += cn * (bn * zre) - cs * (bs * zim);
        dpy += cs * (bs * zre) + cn * (bn * zim);
        dpx_x += cn * bn * ar - cs * bs * ai;
        dpx_y -= cn * bn * ai + cs * bs * ar;
        dpy_x += cs * bs * ar + cn * bn * ai;
        dpy_y += cn * bn * ar - cs * bs * ai;
        // d cos(a - k tau) / d tau = k sin(a - k tau)
        dpx_t += k * (sn * (bn * zre) - ss * (bs * zim));
        dpy_t += k * (ss * (bs * zre) + sn * (bn * zim));
        pre = zre;
        pim = zim;
        double const zret = zre * x - zim * y;
        zim = zim * x + zre * y;
        zre = zret;
        double const br = (kk + 1) * pre, bi = (kk + 1) * pim;
        dptr += sn * (bn * zre) - ss * (bs * zim);
        dptr_x += sn * bn * br - ss * bs * bi;
        dptr_y -= sn * bn * bi + ss * bs * br;
        // d sin(a - k tau) / d tau = -k cos(a - k tau)
        dptr_t -= k * (cn * (bn * zre) - cs * (bs * zim));
    }
    double sc, cc;
    sincos(lag * DEG2RAD_C - ktau, &sc, &cc);
    double const q = s.q;
    double const E = q * (voltage * sc) - q * ((k * s.p0c) * dptr);
    double const E_x = -q * (k * s.p0c) * dptr_x, E_y = -q * (k * s.p0c) * dptr_y;
    double const E_t = -q * voltage * cc * k - q * (k * s.p0c) * dptr_t;
    // kicks: px_out = px_in - chi dpx, py_out = py_in + chi dpy
    s.px += chi * dpx;
    s.py -= chi * dpy;
    double const lpx = l.px, lpy = l.py;
    double const lE = reverse_add_energy(s, l, E / s.energy0) / s.energy0;
    l.x += -chi * lpx * dpx_x + chi * lpy * dpy_x + lE * E_x;
    l.y += -chi * lpx * dpx_y + chi * lpy * dpy_y + lE * E_y;
    add_tau_adjoint(s, l, -chi * lpx * dpx_t + chi * lpy * dpy_t + lE * E_t);
    refresh_lz(s, l);
}

// The space-charge and 4D beam-beam kicks (be_beamfields/track.h:89-337).
__device__ __forceinline__ void reverse_beam_field_impl(RState &s, Lam &l, const uint64_t *rec,
                                                        uint32_t op, uint32_t aux)
{
    const uint64_t *c = rec + 1;
    double const beta0 = s.beta0, rvv = s.rvv;
    if (op == OP_BB4D) {  // :89-149; c: q_part N sigma_x sigma_y beta_s msd Dx Dy Dpx Dpy
        double const ch = 1. * s.q0 * kQelemD;  // qratio = 1 (track.h:121)
        double const beta = beta0 / rvv, bs = W(c[4]);
        double const A = s.chi * W(c[1]) * W(c[0]) * ch / (s.p0c * kQelemD);
        double const K = A * (1. + beta * bs) / (beta + bs);
        double const dK_dbeta = A * (bs * bs - 1.0) / ((beta + bs) * (beta + bs));
        double const dK_dd = dK_dbeta * (-beta0 / (rvv * rvv)) * s.drvv;
        FieldJ const f = field_jacobian(s.x - W(c[6]), s.y - W(c[7]), W(c[2]), W(c[3]), W(c[5]));
        reverse_field_kick(s, l, f, K, dK_dd, 0.0, W(c[8]), W(c[9]));
        return;
    }
    double const charge = kCharge0SiD * s.q0;
    double const pc0 = s.p0c * kCharge0SiD;
    if (op == OP_SC_COASTING) {  // :154-198; c: N C sigma_x sigma_y length x_co y_co msd
        double const K = W(c[0]) * W(c[4]) * s.chi * s.cr * charge * charge * (1.0 - beta0 * beta0) /
                         (W(c[1]) * pc0 * beta0 * rvv);
        FieldJ const f = field_jacobian(s.x - W(c[5]), s.y - W(c[6]), W(c[2]), W(c[3]), W(c[7]));
        reverse_field_kick(s, l, f, K, -K / rvv * s.drvv, 0.0, 0.0, 0.0);
        return;
    }
    // K = C0 g(rvv) lambda, g = (1 - beta0^2 rvv) / (beta0 rvv), g' = -1 / (beta0 rvv^2)
    double const g = (1.0 - beta0 * beta0 * rvv) / (beta0 * rvv);
    double const dg = -1.0 / (beta0 * rvv * rvv);
    if (op == OP_SC_QGAUSS) {  // :203-268; c: N blen sigma_x sigma_y length x_co y_co msd q cq
        double const C0 = s.chi * s.cr * W(c[4]) * charge * charge * W(c[0]) / pc0;
        double const z = s.zeta / rvv;
        double dq;
        double const lam =
            q_gauss_d(z, W(c[8]), 1.0 / (sqrt(2.0) * W(c[1])), W(c[9]), &dq);
        double const K = C0 * g * lam;
        double const dK_dz = C0 * g * dq / rvv;
        double const dK_dd = C0 * (dg * lam + g * dq * (-s.zeta / (rvv * rvv))) * s.drvv;
        FieldJ const f = field_jacobian(s.x - W(c[5]), s.y - W(c[6]), W(c[2]), W(c[3]), W(c[7]));
        reverse_field_kick(s, l, f, K, dK_dd, dK_dz, 0.0, 0.0);
    } else {  // OP_SC_INTERP, :273-337; c: N sigma_x sigma_y length x_co y_co fallback msd ...
        double const C0 = s.chi * s.cr * W(c[3]) * W(c[0]) * charge * charge / pc0;
        double const lam = (aux & 1u) ? ldp_interpolate(c, s.zeta) : W(c[6]);
        double const dlam = (aux & 1u) ? ldp_slope(c, s.zeta) : 0.0;
        double const K = C0 * g * lam;
        FieldJ const f = field_jacobian(s.x - W(c[4]), s.y - W(c[5]), W(c[1]), W(c[2]), W(c[7]));
        reverse_field_kick(s, l, f, K, C0 * dg * lam * s.drvv, C0 * g * dlam, 0.0, 0.0);
    }
    refresh_lz(s, l);
}

// Out-of-line entry points take and return the state by value: a reference
// would pin the caller's state to the stack for the whole walk.
struct RevState {
    RState s;
    Lam l;
};

__device__ __noinline__ RevState reverse_rf_multipole(RevState r, const uint64_t *rec, int order)
{
    reverse_rf_multipole_impl(r.s, r.l, rec, order);
    return r;
}

__device__ __noinline__ RevState reverse_beam_field(RevState r, const uint64_t *rec, uint32_t op,
                                                    uint32_t aux)
{
    reverse_beam_field_impl(r.s, r.l, rec, op, aux);
    return r;
}

// 6D beam-beam (be_beamfields/track.h:342-507), reversed stage by stage
// from the output: the shifts (identity Jacobian), the inverse boost (its
// input is the boost of its output), the slices last to first, the boost.
// Each slice leaves sigma, x + S px and y + S py unchanged, so its kick
// F(xb, yb, S) is recomputed from the slice's output -- once, on Dual<3>
// numbers, which also gives dF/d(xb, yb, S) -- and taken back; lambda goes
// through the slice by the chain rule below.  The map does not read rpp or
// rvv; they follow the restored delta.
__device__ __noinline__ RevState reverse_bb6d(RevState r, const uint64_t *rec, int n_slices)
{
    RState &s = r.s;
    Lam &l = r.l;
    const uint64_t *d = rec + 1;
    const uint64_t *np_ = d + 34;
    const uint64_t *xs_ = np_ + n_slices;
    const uint64_t *ys_ = xs_ + n_slices;
    const uint64_t *ss_ = ys_ + n_slices;
    double const q0 = kQelemD * s.q0;
    double const P0 = s.p0c / kClightD * kQelemD;
    double x = s.x + W(d[27]) - W(d[19]) - W(d[21]);
    double px = s.px + W(d[28]) - W(d[22]);
    double y = s.y + W(d[29]) - W(d[20]) - W(d[23]);
    double py = s.py + W(d[30]) - W(d[24]);
    double sg = s.zeta + W(d[31]) - W(d[25]);
    double dl = s.delta + W(d[32]) - W(d[26]);
    double lam[6] = {l.x, l.px, l.y, l.py, l.z, l.d};
    bb6d_boost_t(d + 1, x, px, y, py, sg, dl);  // the inverse boost's input
    {
        double const u[6] = {x, px, y, py, sg, dl};
        bb6d_boost_jt<true>(d + 1, u, lam);
    }
    for (int i = n_slices - 1; i >= 0; --i) {
        double const Ksl = W(np_[i]) * W(d[0]) * q0 / (P0 * kClightD);
        double const Sv = 0.5 * (sg - W(ss_[i]));
        Dual<3> F[3];
        bb6d_slice_kick_dn(d, Ksl, dseed<3>(x + px * Sv - W(xs_[i]), 0),
                           dseed<3>(y + py * Sv - W(ys_[i]), 1), dseed<3>(Sv, 2), F);
        double const Fx = F[0].v, Fy = F[1].v, Fz = F[2].v;
        // the slice's input: x' = x - S Fx, px' = px + Fx, ...,
        // delta' = delta + Fz + (Fx (px + Fx / 2) + Fy (py + Fy / 2)) / 2
        x += Sv * Fx;
        px -= Fx;
        y += Sv * Fy;
        py -= Fy;
        dl = dl - Fz - 0.5 * (Fx * (px + 0.5 * Fx) + Fy * (py + 0.5 * Fy));
        // adjoints of F, then of xb, yb and S, at that input
        double const lx = lam[0], lpx = lam[1], ly = lam[2], lpy = lam[3], ldl = lam[5];
        double const lFx = -Sv * lx + lpx + 0.5 * ldl * (px + Fx);
        double const lFy = -Sv * ly + lpy + 0.5 * ldl * (py + Fy);
        double const lxb = lFx * F[0].d[0] + lFy * F[1].d[0] + ldl * F[2].d[0];
        double const lyb = lFx * F[0].d[1] + lFy * F[1].d[1] + ldl * F[2].d[1];
        double const lS = lFx * F[0].d[2] + lFy * F[1].d[2] + ldl * F[2].d[2] + px * lxb +
                          py * lyb - Fx * lx - Fy * ly;
        lam[0] = lx + lxb;
        lam[1] = lpx + 0.5 * Fx * ldl + Sv * lxb;
        lam[2] = ly + lyb;
        lam[3] = lpy + 0.5 * Fy * ldl + Sv * lyb;
        lam[4] += 0.5 * lS;
    }
    bb6d_inv_boost_t(d + 1, x, px, y, py, sg, dl);  // the boost's input
    {
        double const u[6] = {x, px, y, py, sg, dl};
        bb6d_boost_jt<false>(d + 1, u, lam);
    }
    l.x = lam[0];
    l.px = lam[1];
    l.y = lam[2];
    l.py = lam[3];
    l.z = lam[4];
    l.d = lam[5];
    s.x = x + W(d[19]) + W(d[21]);
    s.px = px + W(d[22]);
    s.y = y + W(d[20]) + W(d[23]);
    s.py = py + W(d[24]);
    s.zeta = sg + W(d[25]);
    s.delta = dl + W(d[26]);
    // NS(Particles_update_delta_value) (particles.h:5459-5496)
    double const db0 = s.delta * s.beta0;
    double const ptb = sqrt(db0 * db0 + 2.0 * db0 * s.beta0 + 1.0) - 1.0;
    double const opd = 1.0 + s.delta;
    s.rvv = opd / (1.0 + ptb);
    s.rpp = 1.0 / opd;
    set_delta_terms(s, l.z);
    return r;
}

// Multipole (be_multipole/track.h:38-112), with the curvature terms only in
// the CURV instantiation: a runtime branch around them is if-converted, and
// predicated-off FP64 instructions still occupy the FP64 pipe.
template <bool CURV>
__device__ __forceinline__ void reverse_multipole(RState &s, Lam &l, const uint64_t *bal, int n,
                                                  const AdjParams &a, int64_t e, bool on)
{
    double const chi = s.chi, x = s.x, y = s.y;
    // curvature words 2n+2.. : hxl, hyl, length, hxl / length, hyl / length
    // (the ratios are 0 without length)
    double const hxl = CURV ? W(bal[2 * n + 2]) : 0.0;
    double const hyl = CURV ? W(bal[2 * n + 3]) : 0.0;
    double const hxl_l = CURV ? W(bal[2 * n + 5]) : 0.0;
    double const hyl_l = CURV ? W(bal[2 * n + 6]) : 0.0;
    double const lpx = l.px, lpy = l.py;
    if (on) {
        double pr, pi, dr, di;
        horner2(bal, n, x, y, pr, pi, dr, di);
        // input from output: the kick (-chi Re P, chi Im P) taken back
        s.px = fma(chi, pr, s.px);
        s.py = fma(-chi, pi, s.py);
        if (CURV) {
            s.zeta -= chi * (y * hyl - x * hxl);
            s.px -= hxl + hxl * s.delta - chi * W(bal[0]) * x * hxl_l;
            s.py -= -(hyl + hyl * s.delta) + chi * W(bal[1]) * y * hyl_l;
        }
        double const clx = chi * lpx, cly = chi * lpy;
        l.x = fma(-clx, dr, fma(cly, di, l.x));
        l.y = fma(clx, di, fma(cly, dr, l.y));
        if (CURV) {
            l.x -= l.z * chi * hxl + clx * W(bal[0]) * hxl_l;
            l.y += l.z * chi * hyl + cly * W(bal[1]) * hyl_l;
            l.d += lpx * hxl - lpy * hyl;
        }
    }
    int32_t const j0 = a.pbeg ? a.pbeg[e] : 0, j1 = a.pbeg ? a.pbeg[e + 1] : 0;
    if (j0 < j1) {  // warp-uniform
        // d(dpx, dpy)/d bal[2k] = chi (-Re z^k, Im z^k); / d bal[2k+1] = chi (Im z^k, Re z^k)
        double const cx = chi * lpx, cy = chi * lpy;
        for (int32_t j = j0; j < j1; ++j) {
            int const k2 = a.pkind[j];
            double g = 0.0;
            if (on && k2 >= 0) {
                int const kk = k2 >> 1;
                double zr = 1.0, zi = 0.0;
                if (kk > 0) {
                    zr = x;
                    zi = y;
                    for (int k = 1; k < kk; ++k) {
                        double const t = fma(zr, x, -zi * y);
                        zi = fma(zr, y, zi * x);
                        zr = t;
                    }
                }
                g = (k2 & 1) ? fma(cx, zi, cy * zr) : fma(-cx, zr, cy * zi);
                if (CURV && k2 == 0) g -= cx * x * hxl_l;
                if (CURV && k2 == 1) g += cy * y * hyl_l;
            }
            add_grad(a, j, g, on);
        }
    }
}

// Restore the input of one element from its output (state s) and apply
// lambda <- J^T lambda at that input.  `on` is false for lanes that do not
// take part (they still join the warp reductions).  The 6D beam-beam
// reverse is compiled in only where BB6D is set: its call site alone costs
// lattices without the element a few percent (registers saved around it).
template <bool BB6D>
__device__ __forceinline__ void reverse_elem(RState &s, Lam &l, const uint64_t *rec,
                                             const AdjParams &a, int64_t e, bool on)
{
    uint64_t const hdr = rec[0];
    uint32_t const op = (uint32_t)(hdr & 0xFF);
    uint32_t const aux = (uint32_t)(hdr >> 32);
    switch (op) {
    case OP_DRIFT: {  // be_drift/track.h:45-67
        if (!on) break;
        // input from output: x -= L rpp px, zeta -= L (rvv - 1 - rpp^2 (px^2 + py^2) / 2)
        double const L = W(rec[1]);
        double const px = s.px, py = s.py;
        double const a_ = L * s.rpp;
        s.x = fma(-a_, px, s.x);
        s.y = fma(-a_, py, s.y);
        double const p2 = fma(py, py, px * px);
        s.zeta = fma(L, fma(s.hr2, p2, -s.rvvm1), s.zeta);
        // lambda: d(out)/d(px, py, delta) with rpp(delta), rvv(delta):
        //   l.px += L rpp (lx - lz rpp px), l.py likewise,
        //   l.d += L (drpp (lx px + ly py - lz rpp (px^2 + py^2)) + lz drvv)
        double const lx = l.x, ly = l.y;
        l.px = fma(a_, fma(-s.lzr, px, lx), l.px);
        l.py = fma(a_, fma(-s.lzr, py, ly), l.py);
        double const s1 = fma(ly, py, lx * px);
        l.d = fma(L, fma(s.drpp, fma(-s.lzr, p2, s1), s.lzdrvv), l.d);
        break;
    }
    case OP_DRIFT_EXACT: {  // be_drift/track.h:71-97
        if (!on) break;
        double const L = W(rec[1]);
        double const px = s.px, py = s.py;
        double const opd = 1.0 + s.delta;
        double const D2 = opd * opd - (px * px + py * py);
        double const D = sqrt(D2);
        double const lpzi = L / D;
        s.x -= px * lpzi;
        s.y -= py * lpzi;
        s.zeta -= s.rvv * L - opd * lpzi;
        double const D3 = D2 * D;
        double const a_px = L * px / D3, a_py = L * py / D3, a_d = -L * opd / D3;
        double const drvv = s.drvv;
        double const lx = l.x, ly = l.y, lz = l.z;
        l.px += lx * (lpzi + px * a_px) + ly * (py * a_px) - lz * opd * a_px;
        l.py += lx * (px * a_py) + ly * (lpzi + py * a_py) - lz * opd * a_py;
        l.d += lx * (px * a_d) + ly * (py * a_d) + lz * (L * drvv - lpzi - opd * a_d);
        break;
    }
    case OP_MULTIPOLE:  // be_multipole/track.h:38-112
        reverse_multipole<false>(s, l, rec + 1, (int)aux, a, e, on);
        break;
    case OP_MULTIPOLE_CURV:
        reverse_multipole<true>(s, l, rec + 1, (int)aux, a, e, on);
        break;
    case OP_CAVITY: {  // be_cavity/track.h:39-67 + particles.h:5255-5297
        double gV = 0.0;
        if (on) {
            double const V = W(rec[1]), kf = W(rec[2]), lag = W(rec[3]);
            // tau = zeta / (beta0 rvv) is unchanged by the map
            double const phase = lag - kf * (s.zeta / (s.beta0 * s.rvv));
            double sph, cph;
            sincos(phase, &sph, &cph);
            double const lP = reverse_add_energy(s, l, s.q * V * sph / s.energy0);
            add_tau_adjoint(s, l, lP * (-s.q * V * cph * kf / s.energy0));
            refresh_lz(s, l);
            gV = lP * s.q * sph / s.energy0;
        }
        if (a.pbeg) {
            for (int32_t j = a.pbeg[e]; j < a.pbeg[e + 1]; ++j)
                add_grad(a, j, a.pkind[j] < 0 ? gV : 0.0, on);
        }
        break;
    }
    case OP_RF_MULTIPOLE:
        if (on) {
            RevState r = reverse_rf_multipole(RevState{s, l}, rec, (int)aux);
            s = r.s;
            l = r.l;
        }
        break;
    case OP_BB4D:
    case OP_SC_COASTING:
    case OP_SC_QGAUSS:
    case OP_SC_INTERP:
        if (on) {
            RevState r = reverse_beam_field(RevState{s, l}, rec, op, aux);
            s = r.s;
            l = r.l;
        }
        break;
    case OP_BB6D:
        if (BB6D && on) {
            RevState r = reverse_bb6d(RevState{s, l}, rec, (int)(aux & BB6D_SLICES));
            s = r.s;
            l = r.l;
        }
        break;
    case OP_XYSHIFT:  // be_xyshift/track.h:38-55
        if (!on) break;
        s.x -= W(rec[1]);
        s.y -= W(rec[2]);
        break;
    case OP_SROTATION: {  // be_srotation/track.h:38-69
        if (!on) break;
        double const cz = W(rec[1]), sz = W(rec[2]);
        double const x = s.x, y = s.y, px = s.px, py = s.py;
        s.x = cz * x - sz * y;
        s.y = sz * x + cz * y;
        s.px = cz * px - sz * py;
        s.py = sz * px + cz * py;
        double const lx = l.x, ly = l.y, lpx = l.px, lpy = l.py;
        l.x = cz * lx - sz * ly;
        l.y = sz * lx + cz * ly;
        l.px = cz * lpx - sz * lpy;
        l.py = sz * lpx + cz * lpy;
        break;
    }
    case OP_DIPEDGE:  // be_dipedge/track.h:37-51
        if (!on) break;
        s.px -= W(rec[1]) * s.x;
        s.py -= W(rec[2]) * s.y;
        l.x += W(rec[1]) * l.px;
        l.y += W(rec[2]) * l.py;
        break;
    default:  // apertures, monitors, no-ops: identity
        break;
    }
}

template <bool BB6D>
__global__ void __launch_bounds__(kAdjThreads, kAdjBlocksPerSm) adjoint_kernel(AdjParams a)
{
    int const acc_words = a.acc == ACC_COLUMNS ? a.slots * kAdjThreads
                          : (a.acc == ACC_CTA ? a.slots : 0);
    for (int j = threadIdx.x; j < acc_words; j += blockDim.x) s_grad[j] = 0.0;
    __syncthreads();
    int64_t const t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int64_t const cnt = *a.count;
    bool const part = t < cnt;
    int64_t const n = a.n;
    int64_t const i = part ? a.idx[t] : 0;
    int64_t const E = a.num_elements;
    RState s{};
    Lam l{0, 0, 0, 0, 0, 0};
    // turns [t_first, t_last] of this particle lie in the range; in turn
    // t_last it went through elements 0..e_last
    int64_t t_first = a.turn_end, t_last = a.turn_begin - 1, e_last = -1;
    if (part) {
        const int64_t *ks = reinterpret_cast<const int64_t *>(a.start);
        const double *d = reinterpret_cast<const double *>(a.end);
        const int64_t *k = reinterpret_cast<const int64_t *>(a.end);
        t_first = ks[19 * n + i] > a.turn_begin ? ks[19 * n + i] : a.turn_begin;
        if (k[20 * n + i] == 1) {
            t_last = a.turn_end - 1;
            e_last = E - 1;
        } else {
            int64_t const at = k[19 * n + i], ae = k[18 * n + i];
            t_last = at < a.turn_end ? at : a.turn_end - 1;
            e_last = ae < E ? ae : E - 1;
        }
        double const p0c = d[4 * n + i], mass0 = d[1 * n + i];
        s.beta0 = d[2 * n + i];
        s.x = d[6 * n + i];
        s.y = d[7 * n + i];
        s.px = d[8 * n + i];
        s.py = d[9 * n + i];
        s.zeta = d[10 * n + i];
        s.delta = d[12 * n + i];
        s.rpp = d[13 * n + i];
        s.rvv = d[14 * n + i];
        s.chi = d[15 * n + i];
        s.q = d[0 * n + i] * d[16 * n + i];
        s.energy0 = sqrt(p0c * p0c + mass0 * mass0);
        s.p0c = p0c;
        s.q0 = d[0 * n + i];
        s.cr = d[16 * n + i];
        l.x = a.lam[0 * n + i];
        l.px = a.lam[1 * n + i];
        l.y = a.lam[2 * n + i];
        l.py = a.lam[3 * n + i];
        l.z = a.lam[4 * n + i];
        l.d = a.lam[5 * n + i];
        set_delta_terms(s, l.z);
    }
    for (int64_t turn = a.turn_end - 1; turn >= a.turn_begin; --turn) {
        bool const act = part && turn >= t_first && turn <= t_last;
        if (!__any_sync(0xFFFFFFFFu, act)) continue;
        long long const mine = act ? (turn == t_last ? e_last : E - 1) : -1;
        long long wl = mine;
        for (int o = 16; o > 0; o >>= 1) {
            long long const v = __shfl_xor_sync(0xFFFFFFFFu, wl, o);
            wl = v > wl ? v : wl;
        }
        for (int64_t e = (int64_t)wl; e >= 0; --e)
            reverse_elem<BB6D>(s, l, a.stream + a.elem_offset[e], a, e, act && e <= mine);
    }
    if (part) {
        a.lam[0 * n + i] = l.x;
        a.lam[1 * n + i] = l.px;
        a.lam[2 * n + i] = l.y;
        a.lam[3 * n + i] = l.py;
        a.lam[4 * n + i] = l.z;
        a.lam[5 * n + i] = l.d;
    }
    __syncthreads();
    if (a.acc == ACC_COLUMNS) {
        for (int j = threadIdx.x; j < a.slots; j += blockDim.x) {
            double sum = 0.0;
            for (int c = 0; c < kAdjThreads; ++c) sum += s_grad[j * kAdjThreads + c];
            if (sum != 0.0) atomicAdd(&a.grad[j], sum);
        }
    } else if (a.acc == ACC_CTA) {
        for (int j = threadIdx.x; j < a.slots; j += blockDim.x)
            if (s_grad[j] != 0.0) atomicAdd(&a.grad[j], s_grad[j]);
    }
}

}  // namespace

}  // namespace stg

using namespace stg;

extern "C" st_track_status_t st_DeviceLattice_adjoint_turns(
    st_DeviceLattice *lat, const void *d_start, const void *d_end, int64_t n,
    int64_t turn_begin, int64_t turn_end, double *d_lam, const int32_t *d_param_begin,
    const int32_t *d_param_kind, const int32_t *d_param_id, int32_t num_slots, double *d_grad,
    void *stream)
{
    DeviceGuard guard;  // the caller's current device is restored on return
    clear_error();
    LatticeLaunchView v;
    if (!device_lattice_view(lat, &v)) {
        set_error("adjoint: invalid lattice");
        return -1;
    }
    uint32_t const no_adjoint = (1u << OP_FAIL) | (1u << OP_FAIL_LOST) | (1u << OP_TRICUB);
    if (v.op_mask & no_adjoint) {
        set_error("adjoint: the lattice contains elements without an adjoint "
                  "(a TriCub, a disabled map or an unknown type)");
        return -1;
    }
    if (turn_end < turn_begin) {
        set_error("adjoint: turn_end < turn_begin");
        return -1;
    }
    if (n <= 0 || v.num_elements == 0 || turn_end == turn_begin) return 0;
    if (!d_start || !d_end || !d_lam ||
        (d_param_begin && (!d_param_kind || !d_param_id || !d_grad || num_slots <= 0))) {
        set_error("adjoint: missing device buffer");
        return -1;
    }
    if (cudaSetDevice(v.device) != cudaSuccess) {
        set_error("adjoint: cudaSetDevice failed");
        return -1;
    }
    uint64_t *scratch = device_scratch(v.device, select_scratch_words(n));
    if (!scratch || !shared_scratch_begin(v.device, stream)) return -1;
    struct ScratchDone {
        int device;
        void *stream;
        ~ScratchDone() { shared_scratch_end(device, stream); }
    } done{v.device, stream};
    int64_t *idx = nullptr, *count = nullptr;
    // alive at turn_begin with turns left before turn_end
    int rc = launch_select(static_cast<const uint64_t *>(d_start), n, 0, n, MODE_UNTIL, turn_end,
                           scratch, &idx, &count, stream);
    if (rc != 0) {
        set_error(std::string("adjoint selection: ") + cudaGetErrorString((cudaError_t)rc));
        return -1;
    }
    AdjParams a{};
    a.stream = v.stream;
    a.elem_offset = v.elem_offset;
    a.num_elements = v.num_elements;
    a.start = static_cast<const uint64_t *>(d_start);
    a.end = static_cast<const uint64_t *>(d_end);
    a.n = n;
    a.turn_begin = turn_begin;
    a.turn_end = turn_end;
    a.idx = idx;
    a.count = count;
    a.lam = d_lam;
    a.pbeg = d_param_begin;
    a.pkind = d_param_kind;
    a.pid = d_param_id;
    a.grad = d_grad;
    a.slots = d_param_begin ? num_slots : 0;
    a.acc = (a.slots > 0 && a.slots <= kMaxColumnSlots) ? ACC_COLUMNS
            : (a.slots > 0 && a.slots <= kMaxSmemSlots ? ACC_CTA : ACC_GLOBAL);
    size_t const smem = a.acc == ACC_COLUMNS ? (size_t)a.slots * kAdjThreads * sizeof(double)
                        : (a.acc == ACC_CTA ? (size_t)a.slots * sizeof(double) : 0);
    if (smem > 48 * 1024) {
        static bool attr_set[64] = {};
        if (v.device >= 0 && v.device < 64 && !attr_set[v.device]) {
            int const lim = (int)((size_t)kMaxColumnSlots * kAdjThreads * 8);
            if (cudaFuncSetAttribute(adjoint_kernel<true>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, lim) !=
                    cudaSuccess ||
                cudaFuncSetAttribute(adjoint_kernel<false>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, lim) !=
                    cudaSuccess) {
                set_error("adjoint: cannot raise the shared-memory limit");
                return -1;
            }
            attr_set[v.device] = true;
        }
    }
    unsigned const blocks = (unsigned)((n + kAdjThreads - 1) / kAdjThreads);
    if (v.op_mask & (1u << OP_BB6D))
        adjoint_kernel<true><<<blocks, kAdjThreads, smem, static_cast<cudaStream_t>(stream)>>>(a);
    else
        adjoint_kernel<false><<<blocks, kAdjThreads, smem, static_cast<cudaStream_t>(stream)>>>(a);
    rc = (int)cudaGetLastError();
    if (rc != 0) {
        set_error(std::string("adjoint launch: ") + cudaGetErrorString((cudaError_t)rc));
        return -1;
    }
    count_launches(4);
    return 0;
}
