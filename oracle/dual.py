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
limits 1 m, be_limit/track.h:54-88), Multipole, Cavity, XYShift, SRotation,
DipoleEdge, LimitRect, LimitEllipse, LimitRectEllipse, BeamMonitor (no-op).
"""

from __future__ import annotations

import numpy as np

from sixtracklib_gb300.beam_elements import (
    BeamMonitor, Cavity, DipoleEdge, Drift, DriftExact, LimitEllipse, LimitRect,
    LimitRectEllipse, Multipole, SRotation, XYShift)
from sixtracklib_gb300.particles import COL

PI = 3.1415926535897932384626433832795028841971693993751  # constants.h
C_LIGHT = 299792458.0


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


def _where(mask, a: Dual, b: Dual) -> Dual:
    return Dual(np.where(mask, a.v, b.v), np.where(mask, a.d, b.d))


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
        self.q = f[COL["q0"]] * f[COL["charge_ratio"]]
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
    """be_cavity/track.h:39-67 and NS(Particles_add_to_energy_value),
    particles.h:5255-5297; `voltage` may be a Dual."""
    deg2rad = PI / 180.0
    k_factor = (2.0 * PI) / C_LIGHT
    beta0 = p.beta0
    tau = p.zeta / (beta0 * p.rvv)
    phase = deg2rad * lag - (k_factor * frequency) * tau
    energy = p.q * voltage * dsin(phase)
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
