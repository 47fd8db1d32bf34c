"""Forward-mode (dual-number) CPU pass of until-turn tracking.

TEST INFRASTRUCTURE ONLY: the oracle for the engine's reverse-mode adjoint
(imported by tests/ and the bench's adjoint check, never by the product
package).

Every quantity is a dual number ``v + sum_k d[k] eps_k`` (numpy arrays over
particles, ``d`` of shape (tangents, n)); the maps below restate the
reference's maps on such numbers, so one pass gives the derivatives of the
final coordinates along every seeded tangent: initial coordinates (x, px, y,
py, zeta, delta, with rpp / rvv following delta as
NS(Particles_update_delta_value) defines them, particles.h:5459-5496) and
element parameters (multipole bal coefficients, cavity voltage).

Loss bookkeeping follows NS(Track_particle_until_turn) (track/track.h and
track.h): a particle stops at the element where an aperture check fails and
keeps the coordinates (and their derivatives) it had there.  Supported
elements: Drift, DriftExact (with the global aperture check after each drift,
limits 1 m, be_limit/track.h:54-88), Multipole, Cavity, RFMultipole, XYShift,
SRotation, DipoleEdge, LimitRect, LimitEllipse, LimitRectEllipse,
BeamBeam4D, BeamBeam6D, SCCoasting, SCQGaussProfile, SCInterpolatedProfile,
BeamMonitor (no-op).  The Faddeeva function's value comes from the C oracle's cerrf; its
derivative is w'(z) = -2 z w(z) + 2 i / sqrt(pi) at that value.
"""

from __future__ import annotations

import numpy as np

import ctypes as C

from sixtracklib_gb300.beam_elements import (
    BeamBeam4D, BeamBeam6D, BeamMonitor, Cavity, DipoleEdge, Drift, DriftExact, LimitEllipse, LimitRect,
    LimitRectEllipse, Multipole, RFMultipole, SCCoasting, SCInterpolatedProfile,
    SCQGaussProfile, SRotation, XYShift)
from sixtracklib_gb300.particles import COL

PI = 3.1415926535897932384626433832795028841971693993751  # constants.h
C_LIGHT = 299792458.0
EPS0 = 8.854187817620e-12
SQRT_PI = 1.7724538509055160272981674833411451827975494561224
QELEM = 1.60217662e-19        # SIXTRL_QELEM (beam-beam)
CHARGE0_SI = 1.602176634e-19  # NS(PhysConst_charge0_si) (space charge)
DEG2RAD_C = 0.0174532925199432957692369076848861271344287188854172546


class Dual:
    """v: (n,) values; d: (k, n) tangents (or (k, 1) for per-element data)."""

    __slots__ = ("v", "d")
    __array_ufunc__ = None  # numpy operands defer to the Dual operators

    def __init__(self, v, d):
        self.v = v
        self.d = d

    @staticmethod
    def _o(o):
        return o if isinstance(o, Dual) else Dual(np.asarray(o, dtype=np.float64), 0.0)

    def __add__(self, o):
        o = self._o(o)
        return Dual(self.v + o.v, self.d + o.d)

    __radd__ = __add__

    def __sub__(self, o):
        o = self._o(o)
        return Dual(self.v - o.v, self.d - o.d)

    def __rsub__(self, o):
        return self._o(o) - self

    def __neg__(self):
        return Dual(-self.v, -self.d)

    def __mul__(self, o):
        o = self._o(o)
        return Dual(self.v * o.v, self.d * o.v + self.v * o.d)

    __rmul__ = __mul__

    def __truediv__(self, o):
        o = self._o(o)
        q = self.v / o.v
        return Dual(q, (self.d - q * o.d) / o.v)

    def __rtruediv__(self, o):
        return self._o(o) / self


def dsqrt(a: Dual) -> Dual:
    r = np.sqrt(a.v)
    return Dual(r, a.d * (0.5 / r))


def dsin(a: Dual) -> Dual:
    return Dual(np.sin(a.v), a.d * np.cos(a.v))


def dexp(a: Dual) -> Dual:
    e = np.exp(a.v)
    return Dual(e, a.d * e)


def dcos(a: Dual) -> Dual:
    return Dual(np.cos(a.v), -a.d * np.sin(a.v))


def dabs(a: Dual) -> Dual:
    sg = np.where(a.v < 0, -1.0, 1.0)
    return Dual(np.abs(a.v), a.d * sg)


def _where(mask, a: Dual, b: Dual) -> Dual:
    return Dual(np.where(mask, a.v, b.v), np.where(mask, a.d, b.d))


_CERRF = None  # vectorised w(z) of the C oracle, set by track_until


def dcerrf(zr: Dual, zi: Dual):
    """w(z) as two Duals: the C oracle's value, derivative -2 z w + 2i/sqrt(pi)."""
    wr, wi = _CERRF(np.broadcast_to(zr.v, np.shape(zr.v)), np.broadcast_to(zi.v, np.shape(zi.v)))
    dr = -2.0 * (zr.v * wr - zi.v * wi)
    di = -2.0 * (zr.v * wi + zi.v * wr) + 2.0 / SQRT_PI
    return Dual(wr, dr * zr.d - di * zi.d), Dual(wi, dr * zi.d + di * zr.d)


def fields_gauss(x: Dual, y: Dual, sigma_x, sigma_y, min_sigma_diff):
    """NS(get_Ex_Ey_Gx_Gy_gauss) without G terms (be_beamfields/
    gauss_fields.h:56-208): (Ex, Ey)."""
    if abs(sigma_x - sigma_y) < min_sigma_diff:
        sigma = 0.5 * (sigma_x + sigma_y)
        r2 = x * x + y * y
        lin = r2.v < 1e-20
        with np.errstate(divide="ignore", invalid="ignore"):
            t_main = (1 - dexp(-0.5 * r2 / (sigma * sigma))) / (2. * PI * EPS0 * r2)
            t_lin = dsqrt(r2) / (2. * PI * EPS0 * sigma)
        t_lin.d = np.where(np.isfinite(t_lin.d), t_lin.d, 0.0)
        t = _where(lin, t_lin, t_main)
        return t * x, t * y
    abx, aby = dabs(x), dabs(y)
    if sigma_x > sigma_y:
        S = np.sqrt(2. * (sigma_x * sigma_x - sigma_y * sigma_y))
        fact = 1. / (2. * EPS0 * SQRT_PI * S)
        eta_re = sigma_y / sigma_x * abx
        eta_im = sigma_x / sigma_y * aby
        wzr, wzi = dcerrf(abx / S, aby / S)
        wer, wei = dcerrf(eta_re / S, eta_im / S)
        e = dexp(-abx * abx / (2 * sigma_x * sigma_x) - aby * aby / (2 * sigma_y * sigma_y))
        ex = fact * (wzi - wei * e)
        ey = fact * (wzr - wer * e)
    elif sigma_x < sigma_y:
        S = np.sqrt(2. * (sigma_y * sigma_y - sigma_x * sigma_x))
        fact = 1. / (2. * EPS0 * SQRT_PI * S)
        eta_re = sigma_x / sigma_y * aby
        eta_im = sigma_y / sigma_x * abx
        wzr, wzi = dcerrf(aby / S, abx / S)
        wer, wei = dcerrf(eta_re / S, eta_im / S)
        e = dexp(-aby * aby / (2 * sigma_y * sigma_y) - abx * abx / (2 * sigma_x * sigma_x))
        ey = fact * (wzi - wei * e)
        ex = fact * (wzr - wer * e)
    else:
        raise ValueError("equal beam sizes outside the round-beam tolerance")
    ex = _where(x.v < 0, -ex, ex)
    ey = _where(y.v < 0, -ey, ey)
    return ex, ey


class DualParticles:
    """x, px, y, py, zeta, delta, rpp, rvv as dual numbers plus the
    reference quantities as plain arrays."""

    FIELDS = ("x", "px", "y", "py", "zeta", "delta", "rpp", "rvv")

    def __init__(self, block: np.ndarray, k: int):
        f = block.view(np.float64)
        i = block.view(np.int64)
        n = block.shape[1]
        self.n, self.k = n, k
        for name in self.FIELDS:
            setattr(self, name, Dual(f[COL[name]].copy(), np.zeros((k, n))))
        self.beta0 = f[COL["beta0"]].copy()
        self.chi = f[COL["chi"]].copy()
        self.q0 = f[COL["q0"]].copy()
        self.charge_ratio = f[COL["charge_ratio"]].copy()
        self.q = f[COL["q0"]] * f[COL["charge_ratio"]]
        self.p0c = f[COL["p0c"]].copy()
        self.energy0 = np.sqrt(f[COL["p0c"]] ** 2 + f[COL["mass0"]] ** 2)
        self.state = i[COL["state"]].copy()
        self.at_turn = i[COL["at_turn"]].copy()
        self.at_element = i[COL["at_element"]].copy()

    def seed_coordinate(self, tangent: int, name: str, scale=1.0):
        """d(name)/d(seed tangent) = scale; delta also moves rpp and rvv."""
        getattr(self, name).d[tangent] += scale
        if name == "delta":
            self.set_delta(self.delta)

    def set_delta(self, d: Dual):
        """NS(Particles_update_delta_value): particles.h:5459-5496."""
        beta0 = self.beta0
        db0 = d * beta0
        ptau_beta0 = dsqrt(db0 * db0 + 2.0 * db0 * beta0 + 1.0) - 1.0
        opd = 1.0 + d
        self.delta = d
        self.rvv = opd / (1.0 + ptau_beta0)
        self.rpp = 1.0 / opd

    def snapshot(self):
        return {name: getattr(self, name) for name in self.FIELDS}

    def restore_where(self, mask, snap):
        """Lanes in `mask` go back to the snapshot (particles already lost)."""
        for name in self.FIELDS:
            setattr(self, name, _where(mask, snap[name], getattr(self, name)))


# ---------------------------------------------------------------- maps
def drift(p: DualParticles, L):
    """be_drift/track.h:45-67."""
    xp = p.px * p.rpp
    yp = p.py * p.rpp
    dzeta = p.rvv - (1.0 + (xp * xp + yp * yp) * 0.5)
    p.x = p.x + xp * L
    p.y = p.y + yp * L
    p.zeta = p.zeta + L * dzeta


def drift_exact(p: DualParticles, L):
    """be_drift/track.h:71-97."""
    opd = p.delta + 1.0
    lpzi = L / dsqrt(opd * opd - (p.px * p.px + p.py * p.py))
    dzeta = p.rvv * L - opd * lpzi
    p.x = p.x + p.px * lpzi
    p.y = p.y + p.py * lpzi
    p.zeta = p.zeta + dzeta


def multipole(p: DualParticles, order, bal, hxl, hyl, length):
    """be_multipole/track.h:38-112; `bal` is a list of Dual coefficients."""
    x, y, chi = p.x, p.y, p.chi
    dpx, dpy = bal[2 * order], bal[2 * order + 1]
    for k in range(order - 1, -1, -1):
        zre = dpx * x - dpy * y
        zim = dpx * y + dpy * x
        dpx = bal[2 * k] + zre
        dpy = bal[2 * k + 1] + zim
    dpx = -chi * dpx
    dpy = chi * dpy
    if hxl != 0.0 or hyl != 0.0:
        hxlx = x * hxl
        hyly = y * hyl
        p.zeta = p.zeta + chi * (hyly - hxlx)
        dpx = dpx + (hxl + hxl * p.delta)
        dpy = dpy - (hyl + hyl * p.delta)
        if length > 0.0:
            dpx = dpx - chi * bal[0] * hxlx / length
            dpy = dpy + chi * bal[1] * hyly / length
    p.px = p.px + dpx
    p.py = p.py + dpy


def cavity(p: DualParticles, voltage, frequency, lag):
    """be_cavity/track.h:39-67; `voltage` may be a Dual."""
    deg2rad = PI / 180.0
    k_factor = (2.0 * PI) / C_LIGHT
    beta0 = p.beta0
    tau = p.zeta / (beta0 * p.rvv)
    phase = deg2rad * lag - (k_factor * frequency) * tau
    add_energy(p, p.q * voltage * dsin(phase))


def add_energy(p: DualParticles, energy):
    """NS(Particles_add_to_energy_value), particles.h:5255-5297."""
    beta0 = p.beta0
    db0 = p.delta * beta0
    ptau_beta0 = energy / p.energy0 + dsqrt(db0 * db0 + 2.0 * db0 * beta0 + 1.0) - 1.0
    ptau = ptau_beta0 / beta0
    psigma = ptau / beta0
    delta = dsqrt(ptau * ptau + 2.0 * psigma + 1.0) - 1.0
    opd = delta + 1.0
    rvv = opd / (1.0 + ptau_beta0)
    p.delta = delta
    p.zeta = p.zeta * (rvv / p.rvv)
    p.rvv = rvv
    p.rpp = 1.0 / opd


def rf_multipole(p: DualParticles, obj):
    """be_rfmultipole/track.h:39-118."""
    order = int(obj.order)
    bal = np.asarray(obj.bal)
    phase = np.asarray(obj.phase)
    deg2rad = PI / 180.0
    k = float(obj.frequency) * (2.0 * PI) / C_LIGHT
    x, y = p.x, p.y
    q = p.q * 1.0
    ktau = k * p.zeta / (p.beta0 * p.rvv)
    dpx = dpy = dptr = 0.0
    zre, zim = 1.0, 0.0
    for kk in range(order + 1):
        pn = DEG2RAD_C * float(phase[2 * kk]) - ktau
        ps = deg2rad * float(phase[2 * kk + 1]) - ktau
        bn, bs = float(bal[2 * kk]), float(bal[2 * kk + 1])
        cn, cs, sn, ss = dcos(pn), dcos(ps), dsin(pn), dsin(ps)
        dpx = dpx + (cn * (bn * zre) - cs * (bs * zim))
        dpy = dpy + (cs * (bs * zre) + cn * (bn * zim))
        zret = zre * x - zim * y
        zim = zim * x + zre * y
        zre = zret
        dptr = dptr + (sn * (bn * zre) - ss * (bs * zim))
    cav = q * (float(obj.voltage) * dsin(float(obj.lag) * DEG2RAD_C - ktau))
    rfm = -q * ((k * p.p0c) * dptr)
    p.px = p.px + (-p.chi * dpx)
    p.py = p.py + p.chi * dpy
    add_energy(p, cav + rfm)


def beam_beam_4d(p: DualParticles, d):
    """be_beamfields/track.h:89-149 (qratio = 1)."""
    if not d[10] > 0.:
        return
    charge = 1. * p.q0 * QELEM
    x = p.x - d[6]
    y = p.y - d[7]
    beta = p.beta0 / p.rvv
    p0c = p.p0c * QELEM
    ex, ey = fields_gauss(x, y, d[2], d[3], d[5])
    fk = p.chi * d[1] * d[0] * charge * (1. + beta * d[4]) / (p0c * (beta + d[4]))
    p.px = p.px + (fk * ex - d[8])
    p.py = p.py + (fk * ey - d[9])


def _const(val, like: Dual) -> Dual:
    return Dual(np.broadcast_to(np.asarray(val, dtype=np.float64), like.v.shape).copy(),
                np.zeros_like(like.d))


def _sgn(v):
    """(a >= 0) - (a < 0) of the value."""
    return (v >= 0).astype(np.float64) - (v < 0).astype(np.float64)


def _sqrt0(a: Dual) -> Dual:
    """sqrt with derivative 0 where the value is 0: the rotation angle's
    cos / sin at an uncoupled beam, where the tangent of the argument is 0
    or rounding noise."""
    r = np.sqrt(a.v)
    with np.errstate(divide="ignore"):
        g = np.where(r > 0, 0.5 / np.where(r > 0, r, 1.0), 0.0)
    return Dual(r, a.d * g)


def _masked(a: Dual, m, fill) -> Dual:
    return Dual(np.where(m, a.v, fill), np.where(m, a.d, 0.0))


def _ell_fields(a: Dual, b: Dual, sa: Dual, sb: Dual):
    """Elliptic-beam field (E_a, E_b) at |a|, |b| >= 0 for sa > sb
    (gauss_fields.h:56-208, the two orientations are this with a <-> b)."""
    S = dsqrt(2. * (sa * sa - sb * sb))
    fact = 1. / (2. * EPS0 * SQRT_PI * S)
    eta_re = sb / sa * a
    eta_im = sa / sb * b
    wzr, wzi = dcerrf(a / S, b / S)
    wer, wei = dcerrf(eta_re / S, eta_im / S)
    e = dexp(-a * a / (2 * sa * sa) - b * b / (2 * sb * sb))
    return fact * (wzi - wei * e), fact * (wzr - wer * e)


def fields_gauss_g(x: Dual, y: Dual, sigma_x: Dual, sigma_y: Dual, min_sigma_diff):
    """NS(get_Ex_Ey_Gx_Gy_gauss) with the G terms and per-particle beam sizes
    (be_beamfields/gauss_fields.h:56-208): (Ex, Ey, Gx, Gy).  Every branch is
    evaluated on all particles (the elliptic ones on masked, harmless
    arguments) and the particle's own branch is selected."""
    with np.errstate(all="ignore"):
        rnd = np.abs(sigma_x.v - sigma_y.v) < min_sigma_diff
        sigma = 0.5 * (sigma_x + sigma_y)
        r2 = x * x + y * y
        t_lin = dsqrt(r2) / (2. * PI * EPS0 * sigma)
        t_main = (1 - dexp(-0.5 * r2 / (sigma * sigma))) / (2. * PI * EPS0 * r2)
        t = _where(r2.v < 1e-20, t_lin, t_main)
        ex_r, ey_r = t * x, t * y
        eg = dexp(-(x * x + y * y) / (2. * sigma * sigma))
        c = 1. / (2 * PI * EPS0 * sigma * sigma)
        gx_r = 1 / (2. * (x * x + y * y)) * (y * ey_r - x * ex_r + c * x * x * eg)
        gy_r = 1. / (2 * (x * x + y * y)) * (x * ex_r - y * ey_r + c * y * y * eg)
        abx, aby = dabs(x), dabs(y)
        gt = ~rnd & (sigma_x.v > sigma_y.v)
        lt = ~rnd & (sigma_x.v < sigma_y.v)
        ex_g, ey_g = _ell_fields(_masked(abx, gt, 0.0), _masked(aby, gt, 0.0),
                                 _masked(sigma_x, gt, 2.0), _masked(sigma_y, gt, 1.0))
        ey_l, ex_l = _ell_fields(_masked(aby, lt, 0.0), _masked(abx, lt, 0.0),
                                 _masked(sigma_y, lt, 2.0), _masked(sigma_x, lt, 1.0))
        ex_e, ey_e = _where(gt, ex_g, ex_l), _where(gt, ey_g, ey_l)
        ex_e = _where(x.v < 0, -ex_e, ex_e)
        ey_e = _where(y.v < 0, -ey_e, ey_e)
        s11, s33 = sigma_x * sigma_x, sigma_y * sigma_y
        eg = dexp(-x * x / (2 * s11) - y * y / (2 * s33))
        k = 1. / (2 * PI * EPS0)
        gx_e = -1. / (2 * (s11 - s33)) * (x * ex_e + y * ey_e + k * (sigma_y / sigma_x * eg - 1.))
        gy_e = 1. / (2 * (s11 - s33)) * (x * ex_e + y * ey_e + k * (sigma_x / sigma_y * eg - 1.))
    return (_where(rnd, ex_r, ex_e), _where(rnd, ey_r, ey_e), _where(rnd, gx_r, gx_e),
            _where(rnd, gy_r, gy_e))


def bb6d_sigma(sg, S: Dual, thr):
    """NS(BeamBeam6D_propagate_Sigma_matrix) (be_beamfields.h:2232-2385) on
    Duals, branches chosen per particle: (Sig_11_hat, Sig_33_hat, cos theta,
    sin theta and their derivatives along S)."""
    S11_0, S12_0, S13_0, S14_0, S22_0, S23_0, S24_0, S33_0, S34_0, S44_0 = [float(v) for v in sg]
    S11 = S11_0 + 2. * S12_0 * S + S22_0 * S * S
    S33 = S33_0 + 2. * S34_0 * S + S44_0 * S * S
    S13 = S13_0 + (S14_0 + S23_0) * S + S24_0 * S * S
    S12 = S12_0 + S22_0 * S
    S14 = S14_0 + S24_0 * S
    S23 = S23_0 + S24_0 * S
    S34 = S34_0 + S44_0 * S
    S22, S24, S44 = S22_0, S24_0, S44_0
    R = S11 - S33
    Wv = S11 + S33
    T = R * R + 4 * S13 * S13
    dS_R = 2. * (S12_0 - S34_0) + 2 * S * (S22_0 - S44_0)
    dS_W = 2. * (S12_0 + S34_0) + 2 * S * (S22_0 + S44_0)
    dS_S13 = S14_0 + S23_0 + 2 * S24_0 * S
    dS_T = 2 * R * dS_R + 8. * S13 * dS_S13
    signR = _sgn(R.v)
    zero = _const(0.0, S)
    with np.errstate(all="ignore"):
        # T >= thr
        sqrtT = _sqrt0(T)
        c2t = signR * R / sqrtT
        ct_c = _sqrt0(0.5 * (1. + c2t))
        st_c = signR * _sgn(S13.v) * _sqrt0(0.5 * (1. - c2t))
        s11_c = 0.5 * (Wv + signR * sqrtT)
        s33_c = 0.5 * (Wv - signR * sqrtT)
        dc2t = signR * (dS_R / sqrtT - R / (2 * sqrtT * sqrtT * sqrtT) * dS_T)
        dct_c = 1. / (4. * ct_c) * dc2t
        dst_c = _where(np.abs(st_c.v) < thr, (S14 + S23) / R, -1. / (4. * st_c) * dc2t)
        ds11_c = 0.5 * (dS_W + signR * 0.5 / sqrtT * dS_T)
        ds33_c = 0.5 * (dS_W - signR * 0.5 / sqrtT * dS_T)
        # T < thr
        a = S12 - S34
        b = S22 - S44
        c = S14 + S23
        dd = S24
        sq = _sqrt0(a * a + c * c)
        flat = sq.v * sq.v * sq.v < thr
        # ... with a = c = 0: a fixed rotation
        c2 = abs(b) / np.sqrt(b * b + 4 * dd * dd) if abs(dd) > thr else 1.
        ct_a = _const(np.sqrt(0.5 * (1. + c2)), S)
        st_a = _const(float(_sgn(np.float64(b))) * float(_sgn(np.float64(dd))) *
                      np.sqrt(0.5 * (1. - c2)), S)
        # ... otherwise
        c2t_b = dabs(2. * a) / (2 * sq)
        ct_b = _sqrt0(0.5 * (1. + c2t_b))
        sa = _sgn(a.v)
        st_b = sa * _sgn(c.v) * _sqrt0(0.5 * (1. - c2t_b))
        dc2t_b = sa * (0.5 * b / sq - a * (a * b + 2. * c * dd) / (2. * sq * sq * sq))
        dct_b = 1. / (4. * ct_b) * dc2t_b
        dst_b = _where(np.abs(st_b.v) > thr, -1. / (4. * st_b) * dc2t_b, dd / (2. * a))
        s_ab = 0.5 * Wv
        ds11_ab = 0.5 * dS_W
        ds11_b = 0.5 * dS_W + sa * sq
        ds33_b = 0.5 * dS_W - sa * sq
    sing = T.v < thr
    A, B = sing & flat, sing & ~flat

    def pick(va, vb, vc):
        return _where(A, va, _where(B, vb, vc))

    return (pick(s_ab, s_ab, s11_c), pick(s_ab, s_ab, s33_c), pick(ct_a, ct_b, ct_c),
            pick(st_a, st_b, st_c), pick(ds11_ab, ds11_b, ds11_c),
            pick(ds11_ab, ds33_b, ds33_c), pick(zero, dct_b, dct_c), pick(zero, dst_b, dst_c))


def _bb6d_boost(b, x, px, y, py, sg, dl):
    """NS(BeamBeam6D_boost), be_beamfields.h:2101-2160."""
    sphi, cphi, tphi, salpha, calpha = b
    h = dl + 1. - dsqrt((1. + dl) * (1. + dl) - px * px - py * py)
    px_st = px / cphi - h * calpha * tphi / cphi
    py_st = py / cphi - h * salpha * tphi / cphi
    dl_st = dl - px * calpha * tphi - py * salpha * tphi + h * tphi * tphi
    pz_st = dsqrt((1. + dl_st) * (1. + dl_st) - px_st * px_st - py_st * py_st)
    hx = px_st / pz_st
    hy = py_st / pz_st
    hs = 1. - (dl_st + 1) / pz_st
    L11 = 1. + hx * calpha * sphi
    L12 = hx * salpha * sphi
    L13 = calpha * tphi
    L21 = hy * calpha * sphi
    L22 = 1. + hy * salpha * sphi
    L23 = salpha * tphi
    L31 = hs * calpha * sphi
    L32 = hs * salpha * sphi
    L33 = 1. / cphi
    return (L11 * x + L12 * y + L13 * sg, px_st, L21 * x + L22 * y + L23 * sg, py_st,
            L31 * x + L32 * y + L33 * sg, dl_st)


def _bb6d_inv_boost(b, x, px, y, py, sg, dl):
    """NS(BeamBeam6D_inv_boost), be_beamfields.h:2162-2230."""
    sphi, cphi, tphi, salpha, calpha = b
    pz = dsqrt((1. + dl) * (1. + dl) - px * px - py * py)
    hx = px / pz
    hy = py / pz
    hs = 1. - (dl + 1) / pz
    Det = 1. / cphi + (hx * calpha + hy * salpha - hs * sphi) * tphi
    Li11 = (1. / cphi + salpha * tphi * (hy - hs * salpha * sphi)) / Det
    Li12 = (salpha * tphi * (hs * calpha * sphi - hx)) / Det
    Li13 = -tphi * (calpha - hx * salpha * salpha * sphi + hy * calpha * salpha * sphi) / Det
    Li21 = (calpha * tphi * (-hy + hs * salpha * sphi)) / Det
    Li22 = (1. / cphi + calpha * tphi * (hx - hs * calpha * sphi)) / Det
    Li23 = -tphi * (salpha - hy * calpha * calpha * sphi + hx * calpha * salpha * sphi) / Det
    Li31 = -hs * calpha * sphi / Det
    Li32 = -hs * salpha * sphi / Det
    Li33 = (1. + hx * calpha * sphi + hy * salpha * sphi) / Det
    xi = Li11 * x + Li12 * y + Li13 * sg
    yi = Li21 * x + Li22 * y + Li23 * sg
    si = Li31 * x + Li32 * y + Li33 * sg
    h = (dl + 1. - pz) * cphi * cphi
    pxi = px * cphi + h * calpha * tphi
    pyi = py * cphi + h * salpha * tphi
    dli = dl + pxi * calpha * tphi + pyi * salpha * tphi - h * tphi * tphi
    return xi, pxi, yi, pyi, si, dli


def beam_beam_6d(p: DualParticles, words):
    """be_beamfields/track.h:342-507 (payload be_beamfields.h:222-250):
    shift, boost, the strong beam's slices, inverse boost, shift back."""
    d = np.asarray(words, dtype=np.float64)
    if not d[33] > 0.:
        return
    w = d.view(np.uint64)
    ns = int(np.int64(w[18]))

    def rel(f):  # relative-offset array of the payload
        o = int(f + int(w[f]) + 1)
        return d[o:o + ns]

    n_part, x_sl, y_sl, s_sl = rel(34), rel(35), rel(36), rel(37)
    b = [float(v) for v in d[1:6]]
    q0 = QELEM * p.q0
    P0 = p.p0c / C_LIGHT * QELEM
    x, px, y, py, sg, dl = _bb6d_boost(
        b, p.x - d[21] - d[19], p.px - d[22], p.y - d[23] - d[20], p.py - d[24],
        p.zeta - d[25], p.delta - d[26])
    for i in range(ns):
        Ksl = n_part[i] * d[0] * q0 / (P0 * C_LIGHT)
        S = 0.5 * (sg - s_sl[i])
        s11h, s33h, ct, st, ds11h, ds33h, dct, dst = bb6d_sigma(d[6:16], S, d[17])
        xb = x + px * S - x_sl[i]
        yb = y + py * S - y_sl[i]
        xbh = xb * ct + yb * st
        ybh = -xb * st + yb * ct
        dxbh = xb * dct + yb * dst
        dybh = -xb * dst + yb * dct
        ex, ey, gx, gy = fields_gauss_g(xbh, ybh, dsqrt(s11h), dsqrt(s33h), d[16])
        Fxh = Ksl * ex
        Fyh = Ksl * ey
        Gxh = Ksl * gx
        Gyh = Ksl * gy
        Fx = Fxh * ct - Fyh * st
        Fy = Fxh * st + Fyh * ct
        Fz = 0.5 * (Fxh * dxbh + Fyh * dybh + Gxh * ds11h + Gyh * ds33h)
        dl = dl + Fz + 0.5 * (Fx * (px + 0.5 * Fx) + Fy * (py + 0.5 * Fy))
        x = x - S * Fx
        px = px + Fx
        y = y - S * Fy
        py = py + Fy
    x, px, y, py, sg, dl = _bb6d_inv_boost(b, x, px, y, py, sg, dl)
    p.x = x + d[21] + d[19] - d[27]
    p.px = px + d[22] - d[28]
    p.y = y + d[23] + d[20] - d[29]
    p.py = py + d[24] - d[30]
    p.zeta = sg + d[25] - d[31]
    p.set_delta(dl + d[26] - d[32])


def sc_coasting(p: DualParticles, o):
    """be_beamfields/track.h:154-198."""
    charge = CHARGE0_SI * p.q0
    beta0 = p.beta0
    pc0 = p.p0c * CHARGE0_SI
    fk = (o.number_of_particles * o.length * p.chi * p.charge_ratio * charge * charge *
          (1.0 - beta0 * beta0))
    fk = fk / (o.circumference * pc0 * beta0 * p.rvv)
    ex, ey = fields_gauss(p.x - o.x_co, p.y - o.y_co, o.sigma_x, o.sigma_y, o.min_sigma_diff)
    p.px = p.px + fk * ex
    p.py = p.py + fk * ey


def q_gauss(z: Dual, q, sqrt_beta, cq):
    """NS(Math_q_gauss), internal/math_qgauss.h:114-175."""
    arg = -(sqrt_beta * sqrt_beta * z * z)
    omq = 1.0 - q
    if abs(omq) >= 1e-6:
        u = 1.0 + omq * arg
        neg = u.v < 0.0
        uv = np.where(neg, 0.0, u.v)
        ud = np.where(neg, 0.0, u.d)
        ev = uv ** (1.0 / omq)
        with np.errstate(divide="ignore", invalid="ignore"):
            ed = np.where(uv > 0.0, ud * (ev / uv) / omq, 0.0)
        e = Dual(ev, ed)
    else:
        e = dexp(arg)
    return (sqrt_beta / cq) * e


def sc_qgauss(p: DualParticles, o):
    """be_beamfields/track.h:203-268."""
    charge = CHARGE0_SI * p.q0
    beta0 = p.beta0
    beta = beta0 * p.rvv
    pc0 = p.p0c * CHARGE0_SI
    z = p.zeta / p.rvv
    fk = p.chi * p.charge_ratio * o.length * charge * charge * (1.0 - beta0 * beta)
    fk = fk * o.number_of_particles
    fk = fk * q_gauss(z, o.q_param, 1.0 / (np.sqrt(2.0) * o.bunchlength_rms), o.cq)
    fk = fk / (pc0 * beta)
    ex, ey = fields_gauss(p.x - o.x_co, p.y - o.y_co, o.sigma_x, o.sigma_y, o.min_sigma_diff)
    p.px = p.px + fk * ex
    p.py = p.py + fk * ey


def _read_table(addr):
    """A NS(LineDensityProfileData) at a host address: (method, num_values,
    z0, dz, window, values offset, derivatives offset) -- the window spans
    both arrays (reads outside it give 0, as in the oracle)."""
    w = C.cast(C.c_void_p(int(addr)), C.POINTER(C.c_uint64))
    method, cap, va, da, nv = int(w[0]), int(w[1]), int(w[2]), int(w[3]), int(w[6])
    z0 = C.cast(C.c_void_p(int(addr) + 32), C.POINTER(C.c_double))[0]
    dz = C.cast(C.c_void_p(int(addr) + 40), C.POINTER(C.c_double))[0]
    lo, hi = min(va, da), max(va, da) + cap * 8
    win = np.ctypeslib.as_array(C.cast(C.c_void_p(lo), C.POINTER(C.c_double)),
                                shape=((hi - lo) // 8,)).copy()
    return method, nv, z0, dz, win, (va - lo) // 8, (da - lo) // 8


def _interp(table, z: Dual):
    """NS(LineDensityProfileData_interpolate_value) on Duals."""
    method, nv, z0, dz, win, vo, do = table
    inside = (z.v <= z0 + dz * nv) & (z.v >= z0)
    idx = np.where(inside, ((z.v - z0) / dz).astype(np.int64), 0)

    def rd(off, i):
        k = off + i
        ok = (k >= 0) & (k < win.size)
        return np.where(ok, win[np.clip(k, 0, win.size - 1)], 0.0)

    if method == 0:
        r = rd(vo, idx) + (z - (z0 + dz * idx)) * rd(do, idx)
    elif method == 1:
        t2 = (z0 + dz * (idx + 1) - z) / dz
        t1 = (z - (z0 + dz * idx)) / dz
        r = rd(vo, idx + 1) * t1 + rd(vo, idx) * t2
        r = r - rd(do, idx) * dz * dz * (t2 - t2 * t2 * t2) / 6.0
        r = r - rd(do, idx + 1) * dz * dz * (t1 - t1 * t1 * t1) / 6.0
    else:
        r = Dual(np.zeros_like(z.v), np.zeros_like(z.d))
    zero = Dual(np.zeros_like(z.v), np.zeros_like(z.d))
    return _where(inside, r, zero)


def sc_interpolated(p: DualParticles, o):
    """be_beamfields/track.h:273-337."""
    charge = CHARGE0_SI * p.q0
    beta0 = p.beta0
    beta = beta0 * p.rvv
    pc0 = p.p0c * CHARGE0_SI
    fk = (p.chi * p.charge_ratio * o.length * o.number_of_particles * charge * charge *
          (1.0 - beta0 * beta))
    table = _read_table(o.interpol_data_addr) if o.interpol_data_addr else None
    if table is not None and table[0] != 255 and table[1] > 0:
        fk = fk * _interp(table, p.zeta)
    else:
        fk = fk * o.line_density_prof_fallback
    fk = fk / (pc0 * beta)
    ex, ey = fields_gauss(p.x - o.x_co, p.y - o.y_co, o.sigma_x, o.sigma_y, o.min_sigma_diff)
    p.px = p.px + fk * ex
    p.py = p.py + fk * ey


def srotation(p: DualParticles, cz, sz):
    """be_srotation/track.h:38-69."""
    x, y, px, py = p.x, p.y, p.px, p.py
    p.x = cz * x + sz * y
    p.y = -sz * x + cz * y
    p.px = cz * px + sz * py
    p.py = -sz * px + cz * py


# ------------------------------------------------------------ tracking
def _param_duals(elements, params, k, first_tangent):
    """Per element: its parameter values as Duals, tangent seeded for the
    listed params.  params: (element, kind) with kind = bal index or -1."""
    seeded = {}
    for j, (e, kind) in enumerate(params):
        seeded.setdefault(int(e), []).append((int(kind), first_tangent + j))
    out = {}
    for e, lst in seeded.items():
        obj = elements[e]
        if isinstance(obj, Multipole):
            bal = [Dual(np.float64(b), np.zeros((k, 1))) for b in np.asarray(obj.bal)]
            for kind, t in lst:
                bal[kind].d[t] = 1.0
            out[e] = bal
        elif isinstance(obj, Cavity):
            v = Dual(np.float64(obj.voltage), np.zeros((k, 1)))
            for kind, t in lst:
                v.d[t] = 1.0
            out[e] = v
        else:
            raise TypeError(f"element {e} has no differentiable parameter")
    return out


def track_until(elements, block: np.ndarray, until_turn: int, params=(), x_limit=1.0,
                y_limit=1.0):
    """Dual-number until-turn tracking.

    Tangents 0..5 seed the initial x, px, y, py, zeta, delta of every
    particle; tangent 6 + j seeds parameter j of ``params`` (``(element,
    kind)``, kind a multipole bal index or -1 for a cavity voltage).
    Returns ``(values 6 x n, derivatives (6 + m) x 6 x n, state, at_turn,
    at_element)``; rows in the order x, px, y, py, zeta, delta.
    """
    global _CERRF
    if _CERRF is None:
        from oracle.pyoracle import Oracle

        _CERRF = Oracle().cerrf_n
    objs = list(elements.get_elements())
    m = len(params)
    k = 6 + m
    p = DualParticles(block, k)
    for t, name in enumerate(("x", "px", "y", "py", "zeta", "delta")):
        p.seed_coordinate(t, name)
    pduals = _param_duals(objs, params, k, 6)
    active = p.state == 1
    t0 = int(p.at_turn[active].min()) if active.any() else until_turn
    for turn in range(t0, until_turn):
        work = active & (p.at_turn == turn)
        if not work.any():
            continue
        for e, obj in enumerate(objs):
            if not work.any():
                break
            snap = p.snapshot()
            alive = np.ones(p.n, dtype=bool)
            if isinstance(obj, (Drift, DriftExact)):
                (drift if isinstance(obj, Drift) else drift_exact)(p, float(obj.length))
                alive = (np.abs(p.x.v) < x_limit) & (np.abs(p.y.v) < y_limit)
            elif isinstance(obj, Multipole):
                bal = pduals.get(e)
                if bal is None:
                    bal = [np.float64(b) for b in np.asarray(obj.bal)]
                multipole(p, int(obj.order), bal, float(obj.hxl), float(obj.hyl),
                          float(obj.length))
            elif isinstance(obj, Cavity):
                v = pduals.get(e, float(obj.voltage))
                cavity(p, v, float(obj.frequency), float(obj.lag))
            elif isinstance(obj, XYShift):
                p.x = p.x - float(obj.dx)
                p.y = p.y - float(obj.dy)
            elif isinstance(obj, SRotation):
                srotation(p, float(obj.cos_z), float(obj.sin_z))
            elif isinstance(obj, DipoleEdge):
                p.px = p.px + float(obj.r21) * p.x
                p.py = p.py + float(obj.r43) * p.y
            elif isinstance(obj, LimitRect):
                x, y = p.x.v, p.y.v
                alive = ((x >= obj.min_x) & (x <= obj.max_x) & (y >= obj.min_y) &
                         (y <= obj.max_y))
            elif isinstance(obj, LimitEllipse):
                x, y = p.x.v, p.y.v
                alive = (x * x) * obj.b_squ + (y * y) * obj.a_squ <= obj.a_b_squ
            elif isinstance(obj, LimitRectEllipse):
                x, y = p.x.v, p.y.v
                t = x * x * obj.b_squ + y * y * obj.a_squ
                alive = ((x <= obj.max_x) & (x >= -obj.max_x) & (y <= obj.max_y) &
                         (y >= -obj.max_y) & (t <= obj.a_b_squ))
            elif isinstance(obj, RFMultipole):
                rf_multipole(p, obj)
            elif isinstance(obj, BeamBeam4D):
                beam_beam_4d(p, [float(v) for v in np.asarray(obj.data)])
            elif isinstance(obj, BeamBeam6D):
                beam_beam_6d(p, np.asarray(obj.data))
            elif isinstance(obj, SCCoasting):
                sc_coasting(p, obj)
            elif isinstance(obj, SCQGaussProfile):
                sc_qgauss(p, obj)
            elif isinstance(obj, SCInterpolatedProfile):
                sc_interpolated(p, obj)
            elif isinstance(obj, BeamMonitor):
                pass
            else:
                raise NotImplementedError(f"no dual-number map for {type(obj).__name__}")
            # lanes without work keep their state
            p.restore_where(~work, snap)
            lost = work & ~alive
            p.state[lost] = 0
            p.at_element[lost] = e
            work = work & alive
        p.at_turn[work] += 1
        p.at_element[work] = 0
        active = p.state == 1
    names = ("x", "px", "y", "py", "zeta", "delta")
    vals = np.stack([getattr(p, nm).v for nm in names])
    ders = np.stack([getattr(p, nm).d for nm in names], axis=1)  # (k, 6, n)
    return vals, ders, p.state, p.at_turn, p.at_element
