// dual.cuh -- forward-mode dual numbers for element Jacobians in the
// reverse sweep.
//
// A Dual<K> carries a value and its derivatives along K tangents.  The
// adjoint of the 6D beam-beam element uses Dual<3> numbers for the parts
// that have no compact hand-written transpose: a slice's kick as a function
// of (xb, yb, S) -- through the sigma-matrix propagation and the Gaussian
// field with its G terms -- and the Jacobians of the boosts (two passes of
// three of the six coordinates).  Three tangents keep these out-of-line
// functions within the calling kernel's register budget.
//
// Rules: sqrt has derivative 0 where its value is 0 (the rotation angle of
// an uncoupled strong beam, where the argument's tangent is 0 or rounding
// noise); fabs and sign tests use the value; the Faddeeva function's
// derivative is w'(z) = -2 z w(z) + 2 i / sqrt(pi) at the CERN-algorithm
// value of w.
#pragma once

#include "maps.cuh"

namespace stg {

template <int K>
struct Dual {
    double v;
    double d[K];
};

template <int K>
__device__ __forceinline__ Dual<K> dconst(double v)
{
    Dual<K> r;
    r.v = v;
#pragma unroll
    for (int k = 0; k < K; ++k) r.d[k] = 0.0;
    return r;
}

template <int K>
__device__ __forceinline__ Dual<K> dseed(double v, int j)
{
    Dual<K> r = dconst<K>(v);
#pragma unroll
    for (int k = 0; k < K; ++k) r.d[k] = (k == j) ? 1.0 : 0.0;
    return r;
}

#define DN_LOOP _Pragma("unroll") for (int k = 0; k < K; ++k)

template <int K>
__device__ __forceinline__ Dual<K> operator+(const Dual<K> &a, const Dual<K> &b)
{
    Dual<K> r;
    r.v = a.v + b.v;
    DN_LOOP r.d[k] = a.d[k] + b.d[k];
    return r;
}
template <int K>
__device__ __forceinline__ Dual<K> operator+(const Dual<K> &a, double b)
{
    Dual<K> r = a;
    r.v = a.v + b;
    return r;
}
template <int K>
__device__ __forceinline__ Dual<K> operator+(double a, const Dual<K> &b) { return b + a; }
template <int K>
__device__ __forceinline__ Dual<K> operator-(const Dual<K> &a, const Dual<K> &b)
{
    Dual<K> r;
    r.v = a.v - b.v;
    DN_LOOP r.d[k] = a.d[k] - b.d[k];
    return r;
}
template <int K>
__device__ __forceinline__ Dual<K> operator-(const Dual<K> &a, double b)
{
    Dual<K> r = a;
    r.v = a.v - b;
    return r;
}
template <int K>
__device__ __forceinline__ Dual<K> operator-(const Dual<K> &a)
{
    Dual<K> r;
    r.v = -a.v;
    DN_LOOP r.d[k] = -a.d[k];
    return r;
}
template <int K>
__device__ __forceinline__ Dual<K> operator-(double a, const Dual<K> &b)
{
    Dual<K> r;
    r.v = a - b.v;
    DN_LOOP r.d[k] = -b.d[k];
    return r;
}
template <int K>
__device__ __forceinline__ Dual<K> operator*(const Dual<K> &a, const Dual<K> &b)
{
    Dual<K> r;
    r.v = a.v * b.v;
    DN_LOOP r.d[k] = fma(a.d[k], b.v, a.v * b.d[k]);
    return r;
}
template <int K>
__device__ __forceinline__ Dual<K> operator*(const Dual<K> &a, double b)
{
    Dual<K> r;
    r.v = a.v * b;
    DN_LOOP r.d[k] = a.d[k] * b;
    return r;
}
template <int K>
__device__ __forceinline__ Dual<K> operator*(double a, const Dual<K> &b) { return b * a; }
template <int K>
__device__ __forceinline__ Dual<K> operator/(const Dual<K> &a, const Dual<K> &b)
{
    Dual<K> r;
    r.v = a.v / b.v;
    double const ib = 1.0 / b.v;
    DN_LOOP r.d[k] = (a.d[k] - r.v * b.d[k]) * ib;
    return r;
}
template <int K>
__device__ __forceinline__ Dual<K> operator/(const Dual<K> &a, double b)
{
    Dual<K> r;
    r.v = a.v / b;
    DN_LOOP r.d[k] = a.d[k] / b;
    return r;
}
template <int K>
__device__ __forceinline__ Dual<K> operator/(double a, const Dual<K> &b)
{
    Dual<K> r;
    r.v = a / b.v;
    double const g = -r.v / b.v;
    DN_LOOP r.d[k] = g * b.d[k];
    return r;
}

template <int K>
__device__ __forceinline__ Dual<K> dsqrt(const Dual<K> &a)
{
    Dual<K> r;
    r.v = sqrt(a.v);
    double const g = r.v > 0.0 ? 0.5 / r.v : 0.0;
    DN_LOOP r.d[k] = a.d[k] * g;
    return r;
}
template <int K>
__device__ __forceinline__ Dual<K> dexp(const Dual<K> &a)
{
    Dual<K> r;
    r.v = exp(a.v);
    DN_LOOP r.d[k] = a.d[k] * r.v;
    return r;
}
template <int K>
__device__ __forceinline__ Dual<K> dfabs(const Dual<K> &a) { return a.v < 0.0 ? -a : a; }

// the same expressions on plain doubles and on dual numbers
__device__ __forceinline__ double tsqrt(double a) { return sqrt(a); }
template <int K>
__device__ __forceinline__ Dual<K> tsqrt(const Dual<K> &a) { return dsqrt(a); }

__device__ __forceinline__ double sgn_of(double a) { return (double)((a >= 0) - (a < 0)); }

// w(z) and its derivative along the tangents of z = zr + i zi
template <int K>
static __device__ __noinline__ void cerrf_dn(const Dual<K> &zr, const Dual<K> &zi, Dual<K> &wr, Dual<K> &wi)
{
    double a, b;
    cerrf(zr.v, zi.v, &a, &b);
    double const dr = -2.0 * (zr.v * a - zi.v * b);
    double const di = -2.0 * (zr.v * b + zi.v * a) + 2.0 / kSqrtPiD;
    wr.v = a;
    wi.v = b;
    DN_LOOP
    {
        wr.d[k] = dr * zr.d[k] - di * zi.d[k];
        wi.d[k] = dr * zi.d[k] + di * zr.d[k];
    }
}

// Elliptic field (E_a, E_b) at a = |x|, b = |y| >= 0 for sa > sb
// (gauss_fields.h:56-208; the other orientation is this with a <-> b).
template <int K>
__device__ __forceinline__ void ell_fields_dn(const Dual<K> &a, const Dual<K> &b, const Dual<K> &sa, const Dual<K> &sb,
                                              Dual<K> &ea, Dual<K> &eb)
{
    Dual<K> const S = dsqrt(2. * (sa * sa - sb * sb));
    Dual<K> const fact = 1. / (2. * kEps0D * kSqrtPiD * S);
    Dual<K> const eta_re = sb / sa * a;
    Dual<K> const eta_im = sa / sb * b;
    Dual<K> wzr, wzi, wer, wei;
    cerrf_dn(a / S, b / S, wzr, wzi);
    cerrf_dn(eta_re / S, eta_im / S, wer, wei);
    Dual<K> const e = dexp(-a * a / (2 * sa * sa) - b * b / (2 * sb * sb));
    ea = fact * (wzi - wei * e);
    eb = fact * (wzr - wer * e);
}

// NS(get_Ex_Ey_Gx_Gy_gauss) with the G terms (gauss_fields.h:56-208) on
// Dual<K> numbers: out = (Ex, Ey, Gx, Gy).
template <int K>
static __device__ __noinline__ void fields_gauss_dn(const Dual<K> &x, const Dual<K> &y, const Dual<K> &sigma_x,
                                                    const Dual<K> &sigma_y, double min_sigma_diff,
                                                    Dual<K> *out)
{
    Dual<K> ex, ey, gx, gy;
    if (fabs(sigma_x.v - sigma_y.v) < min_sigma_diff) {
        Dual<K> const sigma = 0.5 * (sigma_x + sigma_y);
        Dual<K> const r2 = x * x + y * y;
        Dual<K> const t = r2.v < 1e-20 ? dsqrt(r2) / (2. * kPiD * kEps0D * sigma)
                                  : (1. - dexp(-0.5 * r2 / (sigma * sigma))) /
                                        (2. * kPiD * kEps0D * r2);
        ex = t * x;
        ey = t * y;
        Dual<K> const eg = dexp(-(x * x + y * y) / (2. * sigma * sigma));
        Dual<K> const c = 1. / (2 * kPiD * kEps0D * sigma * sigma);
        gx = 1 / (2. * (x * x + y * y)) * (y * ey - x * ex + c * x * x * eg);
        gy = 1. / (2 * (x * x + y * y)) * (x * ex - y * ey + c * y * y * eg);
    } else {
        Dual<K> const abx = dfabs(x), aby = dfabs(y);
        if (sigma_x.v > sigma_y.v) {
            ell_fields_dn(abx, aby, sigma_x, sigma_y, ex, ey);
        } else if (sigma_x.v < sigma_y.v) {
            ell_fields_dn(aby, abx, sigma_y, sigma_x, ey, ex);
        } else {
            ex = ey = dconst<K>(__longlong_as_double(0x7FF0000000000000ll));  // 1/0
        }
        if (x.v < 0) ex = -ex;
        if (y.v < 0) ey = -ey;
        Dual<K> const s11 = sigma_x * sigma_x, s33 = sigma_y * sigma_y;
        Dual<K> const eg = dexp(-x * x / (2 * s11) - y * y / (2 * s33));
        double const kk = 1. / (2 * kPiD * kEps0D);
        Dual<K> const xy = x * ex + y * ey;
        gx = -1. / (2 * (s11 - s33)) * (xy + kk * (sigma_y / sigma_x * eg - 1.));
        gy = 1. / (2 * (s11 - s33)) * (xy + kk * (sigma_x / sigma_y * eg - 1.));
    }
    out[0] = ex;
    out[1] = ey;
    out[2] = gx;
    out[3] = gy;
}

// NS(BeamBeam6D_propagate_Sigma_matrix) (be_beamfields.h:2232-2385) on Dual<K>
// numbers: out = (Sig_11_hat, Sig_33_hat, cos theta, sin theta, and their
// derivatives along S).
template <int K>
static __device__ __noinline__ void bb6d_sigma_dn(const uint64_t *sg, const Dual<K> &S, double thr,
                                                  Dual<K> *out)
{
    double const S11_0 = W(sg[0]), S12_0 = W(sg[1]), S13_0 = W(sg[2]), S14_0 = W(sg[3]),
                 S22_0 = W(sg[4]), S23_0 = W(sg[5]), S24_0 = W(sg[6]), S33_0 = W(sg[7]),
                 S34_0 = W(sg[8]), S44_0 = W(sg[9]);
    Dual<K> const S11 = S11_0 + 2. * S12_0 * S + S22_0 * S * S;
    Dual<K> const S33 = S33_0 + 2. * S34_0 * S + S44_0 * S * S;
    Dual<K> const S13 = S13_0 + (S14_0 + S23_0) * S + S24_0 * S * S;
    Dual<K> const S12 = S12_0 + S22_0 * S;
    Dual<K> const S14 = S14_0 + S24_0 * S;
    Dual<K> const S23 = S23_0 + S24_0 * S;
    Dual<K> const S34 = S34_0 + S44_0 * S;
    double const S22 = S22_0, S24 = S24_0, S44 = S44_0;
    Dual<K> const R = S11 - S33;
    Dual<K> const Wv = S11 + S33;
    Dual<K> const T = R * R + 4 * S13 * S13;
    Dual<K> const dS_R = 2. * (S12_0 - S34_0) + 2 * S * (S22_0 - S44_0);
    Dual<K> const dS_W = 2. * (S12_0 + S34_0) + 2 * S * (S22_0 + S44_0);
    Dual<K> const dS_S13 = S14_0 + S23_0 + 2 * S24_0 * S;
    Dual<K> const dS_T = 2 * R * dS_R + 8. * S13 * dS_S13;
    double const signR = sgn_of(R.v);
    Dual<K> s11h, s33h, ct, st, ds11h, ds33h, dct, dst;
    if (T.v < thr) {
        Dual<K> const a = S12 - S34;
        double const b = S22 - S44;
        Dual<K> const c = S14 + S23;
        double const dd = S24;
        Dual<K> const sq = dsqrt(a * a + c * c);
        if (sq.v * sq.v * sq.v < thr) {
            double const c2t = (fabs(dd) > thr) ? fabs(b) / sqrt(b * b + 4 * dd * dd) : 1.;
            ct = dconst<K>(sqrt(0.5 * (1. + c2t)));
            st = dconst<K>(sgn_of(b) * sgn_of(dd) * sqrt(0.5 * (1. - c2t)));
            dct = dconst<K>(0.);
            dst = dconst<K>(0.);
            s11h = 0.5 * Wv;
            s33h = 0.5 * Wv;
            ds11h = 0.5 * dS_W;
            ds33h = 0.5 * dS_W;
        } else {
            Dual<K> const c2t = dfabs(2. * a) / (2 * sq);
            ct = dsqrt(0.5 * (1. + c2t));
            st = sgn_of(a.v) * sgn_of(c.v) * dsqrt(0.5 * (1. - c2t));
            Dual<K> const dc2t = sgn_of(a.v) * (0.5 * b / sq - a * (a * b + 2. * c * dd) /
                                                              (2. * sq * sq * sq));
            dct = 1. / (4. * ct) * dc2t;
            if (fabs(st.v) > thr)
                dst = -1. / (4. * st) * dc2t;
            else
                dst = dd / (2. * a);
            s11h = 0.5 * Wv;
            s33h = 0.5 * Wv;
            ds11h = 0.5 * dS_W + sgn_of(a.v) * sq;
            ds33h = 0.5 * dS_W - sgn_of(a.v) * sq;
        }
    } else {
        Dual<K> const sqrtT = dsqrt(T);
        Dual<K> const c2t = signR * R / sqrtT;
        ct = dsqrt(0.5 * (1. + c2t));
        st = signR * sgn_of(S13.v) * dsqrt(0.5 * (1. - c2t));
        s11h = 0.5 * (Wv + signR * sqrtT);
        s33h = 0.5 * (Wv - signR * sqrtT);
        Dual<K> const dc2t = signR * (dS_R / sqrtT - R / (2 * sqrtT * sqrtT * sqrtT) * dS_T);
        dct = 1. / (4. * ct) * dc2t;
        if (fabs(st.v) < thr)
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

// NS(BeamBeam6D_boost) (be_beamfields.h:2101-2160); b = the payload's
// (sin phi, cos phi, tan phi, sin alpha, cos alpha) words.
template <class T>
__device__ __forceinline__ void bb6d_boost_t(const uint64_t *b, T &x, T &px, T &y, T &py, T &sg,
                                             T &dl)
{
    double const sphi = W(b[0]), cphi = W(b[1]), tphi = W(b[2]), salpha = W(b[3]),
                 calpha = W(b[4]);
    T const h = dl + 1. - tsqrt((1. + dl) * (1. + dl) - px * px - py * py);
    T const px_st = px / cphi - h * calpha * tphi / cphi;
    T const py_st = py / cphi - h * salpha * tphi / cphi;
    T const dl_st = dl - px * calpha * tphi - py * salpha * tphi + h * tphi * tphi;
    T const pz_st = tsqrt((1. + dl_st) * (1. + dl_st) - px_st * px_st - py_st * py_st);
    T const hx = px_st / pz_st;
    T const hy = py_st / pz_st;
    T const hs = 1. - (dl_st + 1) / pz_st;
    T const L11 = 1. + hx * calpha * sphi;
    T const L12 = hx * salpha * sphi;
    double const L13 = calpha * tphi;
    T const L21 = hy * calpha * sphi;
    T const L22 = 1. + hy * salpha * sphi;
    double const L23 = salpha * tphi;
    T const L31 = hs * calpha * sphi;
    T const L32 = hs * salpha * sphi;
    double const L33 = 1. / cphi;
    T const nx = L11 * x + L12 * y + L13 * sg;
    T const ny = L21 * x + L22 * y + L23 * sg;
    T const ns = L31 * x + L32 * y + L33 * sg;
    x = nx;
    y = ny;
    sg = ns;
    px = px_st;
    py = py_st;
    dl = dl_st;
}

// NS(BeamBeam6D_inv_boost) (be_beamfields.h:2162-2230).
template <class T>
__device__ __forceinline__ void bb6d_inv_boost_t(const uint64_t *b, T &x, T &px, T &y, T &py,
                                                 T &sg, T &dl)
{
    double const sphi = W(b[0]), cphi = W(b[1]), tphi = W(b[2]), salpha = W(b[3]),
                 calpha = W(b[4]);
    T const pz = tsqrt((1. + dl) * (1. + dl) - px * px - py * py);
    T const hx = px / pz;
    T const hy = py / pz;
    T const hs = 1. - (dl + 1) / pz;
    T const Det = 1. / cphi + (hx * calpha + hy * salpha - hs * sphi) * tphi;
    T const Li11 = (1. / cphi + salpha * tphi * (hy - hs * salpha * sphi)) / Det;
    T const Li12 = (salpha * tphi * (hs * calpha * sphi - hx)) / Det;
    T const Li13 =
        -tphi * (calpha - hx * salpha * salpha * sphi + hy * calpha * salpha * sphi) / Det;
    T const Li21 = (calpha * tphi * (-hy + hs * salpha * sphi)) / Det;
    T const Li22 = (1. / cphi + calpha * tphi * (hx - hs * calpha * sphi)) / Det;
    T const Li23 =
        -tphi * (salpha - hy * calpha * calpha * sphi + hx * calpha * salpha * sphi) / Det;
    T const Li31 = -hs * calpha * sphi / Det;
    T const Li32 = -hs * salpha * sphi / Det;
    T const Li33 = (1. + hx * calpha * sphi + hy * salpha * sphi) / Det;
    T const xi = Li11 * x + Li12 * y + Li13 * sg;
    T const yi = Li21 * x + Li22 * y + Li23 * sg;
    T const si = Li31 * x + Li32 * y + Li33 * sg;
    T const h = (dl + 1. - pz) * cphi * cphi;
    T const pxi = px * cphi + h * calpha * tphi;
    T const pyi = py * cphi + h * salpha * tphi;
    T const dli = dl + pxi * calpha * tphi + pyi * salpha * tphi - h * tphi * tphi;
    x = xi;
    y = yi;
    sg = si;
    px = pxi;
    py = pyi;
    dl = dli;
}

// One slice of the strong beam (be_beamfields/track.h:418-480) as a
// function of xb = x + px S - x_slice, yb = y + py S - y_slice and
// S = (sigma - sigma_slice) / 2 only: F = (Fx, Fy, Fz), the kicks on px,
// py and delta (Fz without the kinetic term) with the derivatives along
// the tangents of (xb, yb, S).
template <int K>
static __device__ __noinline__ void bb6d_slice_kick_dn(const uint64_t *d, double Ksl,
                                                       const Dual<K> &xb, const Dual<K> &yb,
                                                       const Dual<K> &S, Dual<K> *F)
{
    Dual<K> sm[8];
    bb6d_sigma_dn(d + 6, S, W(d[17]), sm);
    Dual<K> const ct = sm[2], st = sm[3];
    Dual<K> const xbh = xb * ct + yb * st;
    Dual<K> const ybh = -xb * st + yb * ct;
    Dual<K> const dxbh = xb * sm[6] + yb * sm[7];
    Dual<K> const dybh = -xb * sm[7] + yb * sm[6];
    Dual<K> f[4];
    fields_gauss_dn(xbh, ybh, dsqrt(sm[0]), dsqrt(sm[1]), W(d[16]), f);
    Dual<K> const Fxh = Ksl * f[0], Fyh = Ksl * f[1], Gxh = Ksl * f[2], Gyh = Ksl * f[3];
    F[0] = Fxh * ct - Fyh * st;
    F[1] = Fxh * st + Fyh * ct;
    F[2] = 0.5 * (Fxh * dxbh + Fyh * dybh + Gxh * sm[4] + Gyh * sm[5]);
}

// lam <- J^T lam for the boost (INV false) or the inverse boost at the
// point u = (x, px, y, py, sigma, delta): two passes of three tangents.
template <bool INV>
static __device__ __noinline__ void bb6d_boost_jt(const uint64_t *b, const double *u, double *lam)
{
    double out[6];
#pragma unroll
    for (int p = 0; p < 6; p += 3) {
        Dual<3> v[6];
#pragma unroll
        for (int j = 0; j < 6; ++j) v[j] = dseed<3>(u[j], j - p);
        if (INV)
            bb6d_inv_boost_t(b, v[0], v[1], v[2], v[3], v[4], v[5]);
        else
            bb6d_boost_t(b, v[0], v[1], v[2], v[3], v[4], v[5]);
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            double a = 0.0;
#pragma unroll
            for (int i = 0; i < 6; ++i) a = fma(lam[i], v[i].d[k], a);
            out[p + k] = a;
        }
    }
#pragma unroll
    for (int j = 0; j < 6; ++j) lam[j] = out[j];
}

#undef DN_LOOP

}  // namespace stg
