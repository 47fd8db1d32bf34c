"""Algorithmic FP64 operation counts of the element maps.

Frozen per-type table: the number of floating-point operations (add, sub,
mul, div, sqrt and each libm call counted as one; comparisons and sign flips
not counted) that the reference's formula for one particle through one
element performs (sixtracklib/common/be_*/track.h).  A lattice's cost per
particle-element-turn is the table averaged over its elements; the kernel's
achieved FLOP/s is that average times its particle-element-turns per second.
"""

from __future__ import annotations

import numpy as np

from .cbuffer import CBuffer

# drift 15 (+2 for the global aperture |x|,|y| as sign*x, sign*y)
FLOPS_DRIFT = 15 + 2
# exact drift: opd 1, squares/sums 5, sqrt 1, div 1, dzeta 3, x/y 4, s 1, zeta 1 (+2 aperture)
FLOPS_DRIFT_EXACT = 17 + 2
FLOPS_XYSHIFT = 2
FLOPS_SROTATION = 12
FLOPS_LIMIT_ELLIPSE = 5
FLOPS_LIMIT_RECT = 0
FLOPS_LIMIT_RECT_ELLIPSE = 5
FLOPS_DIPEDGE = 4
# add_to_energy 36 + cavity phase/energy 9
FLOPS_CAVITY = 45
# TriCub (be_tricub/track.h:51-224) from per-cell coefficients (an FMA
# counted as 2): grid coordinates z, fx, fy, fz, floor, fractions (17); the
# three partial derivatives of the tricubic as nested Horner forms (per
# (i, j): the z polynomial 6, its z derivative 6, the y sums 4, the y
# derivative 3 for j >= 1; per i: the x sums 7 or 4) (317); scaling by
# length / d and the dipolar corrections (6); the energy kick 3, px / py 2
# and add_to_energy 36.  The reference forms the 64 coefficients per
# particle (1,000 products and 936 sums) and sums the 144 derivative terms
# one by one (720); the coefficients depend only on the grid cell, which
# makes them lattice preparation here (computed once per cell).
FLOPS_TRICUB = 17 + 317 + 6 + 3 + 2 + 36


def multipole_flops(order: int, curvature: bool = False) -> int:
    """Horner: 8 per order step, 4 for the chi scaling and px/py update;
    the curvature branch adds ~14."""
    return 8 * order + 4 + (14 if curvature else 0)


def lattice_flops_per_element(cbuffer: CBuffer) -> float:
    """Average algorithmic FP64 operations per particle per element."""
    tot = 0
    n = 0
    for o in cbuffer.objects:
        t = o.typeid
        w = o.words
        if t == 2:
            f = FLOPS_DRIFT
        elif t == 3:
            f = FLOPS_DRIFT_EXACT
        elif t == 4:
            hxl = w[2:3].view(np.float64)[0]
            hyl = w[3:4].view(np.float64)[0]
            f = multipole_flops(int(w[0]), bool(hxl != 0.0 or hyl != 0.0))
        elif t == 5:
            f = FLOPS_CAVITY
        elif t == 6:
            f = FLOPS_XYSHIFT
        elif t == 7:
            f = FLOPS_SROTATION
        elif t == 11:
            f = FLOPS_LIMIT_RECT
        elif t == 12:
            f = FLOPS_LIMIT_ELLIPSE
        elif t == 16:
            f = FLOPS_LIMIT_RECT_ELLIPSE
        elif t == 24:
            f = FLOPS_DIPEDGE
        elif t == 261:
            f = FLOPS_TRICUB
        else:
            f = 0
        tot += f
        n += 1
    return tot / max(n, 1)


# ------------------------------------------------------------ beam fields
# Counted from the reference's formulas with the same rule (add, sub, mul,
# div, sqrt and each libm call = 1; comparisons, fabs and sign flips = 0).

# cerrf (be_beamfields/faddeeva_cern.h:45-120), CERN algorithm of K. Koelbig:
# inside the rectangle |x| < 5.33, |y| < 4.29 the set-up of q, h, nc, nu,
# xl (14), nu continued-fraction steps of 11 and nc series steps of 8, and
# the final scaling (2); outside it 9 continued-fraction steps (99 + 2).
CERRF_SETUP, CERRF_CF_STEP, CERRF_SERIES_STEP, CERRF_SCALE = 14, 11, 8, 2
CERRF_X_LIM, CERRF_Y_LIM = 5.33, 4.29


def cerrf_flops(re, im):
    """FP64 operations of one reference cerrf(re + i im) call, per point
    (arrays): the iteration counts depend on where z lies."""
    x = np.abs(np.asarray(re, dtype=np.float64))
    y = np.abs(np.asarray(im, dtype=np.float64))
    small = (y < CERRF_Y_LIM) & (x < CERRF_X_LIM)
    xs, ys = np.where(small, x, 0.0), np.where(small, y, 0.0)
    q = (1.0 - ys / CERRF_Y_LIM) * np.sqrt(np.maximum(1.0 - (xs / CERRF_X_LIM) ** 2, 0.0))
    nc = 7 + np.floor(23.0 * q)
    nu = 10 + np.floor(21.0 * q)
    f_small = CERRF_SETUP + CERRF_CF_STEP * nu + CERRF_SERIES_STEP * nc + CERRF_SCALE
    f_large = 9 * CERRF_CF_STEP + CERRF_SCALE
    f = np.where(small, f_small, f_large)
    f = f + np.where(y == 0.0, 2, 0)            # Wx = exp(-x x)
    f = f + np.where(np.asarray(im) < 0.0, 20, 0)  # reflection to y < 0
    return f


# get_Ex_Ey_Gx_Gy_gauss (be_beamfields/gauss_fields.h:153-208): the branch
# test (1); round: sigma (2) + get_transv_field_gauss_round at Delta = 0
# (18); elliptic: Sig_11, Sig_33 (2) + get_transv_field_gauss_ellip (35,
# without its two cerrf calls); the G terms when not skipped: round 52,
# elliptic 50.
FIELD_ROUND = 1 + 2 + 18
FIELD_ELLIPTIC = 1 + 2 + 35
G_ROUND, G_ELLIPTIC = 52, 50

# BeamBeam4D (be_beamfields/track.h:89-149) without the field: charge (2),
# x, y (2), beta (1), p0c (1), fact_kick (10), the two kicks (6).
FLOPS_BB4D_BASE = 22
# SCQGaussProfile (be_beamfields/track.h:203-268) without the field:
# charge, beta, pc0, z (4), fact_kick (7 + 1), Math_q_gauss with its
# sqrt_beta (9, q = 1; 12 otherwise; internal/math_qgauss.h:114-175), the
# product (1), the division by pc0 beta (2), x - x_co, y - y_co (2), kicks (4).
FLOPS_SC_QGAUSS_BASE = 30
FLOPS_SC_QGAUSS_Q_NOT_1 = 3
# SCCoasting (be_beamfields/track.h:154-198) without the field.
FLOPS_SC_COASTING_BASE = 20
# BeamBeam6D (be_beamfields/track.h:342-507, be_beamfields.h:2101-2385)
# per element: charge and P0 (3), frame change (8), boost (73), inverse
# boost (116), back to the lab frame (14), Particles_update_delta_value (14).
FLOPS_BB6D_ELEMENT = 3 + 8 + 73 + 116 + 14 + 14
# per slice without the field: Ksl (4), S (2), Sigma propagation up to the
# branch (59), the transverse coordinates and their S derivatives (18), the
# two sqrt of the sigmas (2), kicks and Hirata's synchro-beam update (34);
# the branch: singular 21, regular 41.
FLOPS_BB6D_SLICE = 4 + 2 + 59 + 18 + 2 + 34
FLOPS_BB6D_SINGULAR, FLOPS_BB6D_REGULAR = 21, 41


def _field_flops(dx, dy, sx, sy, min_sigma_diff, with_g):
    """Mean operations of one get_Ex_Ey_Gx_Gy_gauss call over the points
    (dx, dy) relative to the strong beam's centre."""
    if abs(sx - sy) < min_sigma_diff:
        return FIELD_ROUND + (G_ROUND if with_g else 0)
    ax, ay = np.abs(dx), np.abs(dy)
    if sx > sy:
        s = np.sqrt(2.0 * (sx * sx - sy * sy))
        zeta, eta = (ax / s, ay / s), (sy / sx * ax / s, sx / sy * ay / s)
    else:
        s = np.sqrt(2.0 * (sy * sy - sx * sx))
        zeta, eta = (ay / s, ax / s), (sx / sy * ay / s, sy / sx * ax / s)
    w = float(np.mean(cerrf_flops(*zeta) + cerrf_flops(*eta)))
    return FIELD_ELLIPTIC + (G_ELLIPTIC if with_g else 0) + w


def element_flops(obj, x=None, y=None) -> float:
    """Algorithmic FP64 operations of one particle through element `obj` (a
    beam_elements object).  For the elliptic Gaussian fields the cost of the
    Faddeeva function depends on the particle's position relative to the
    strong beam: it is averaged over the positions (x, y) given, without the
    element's own offsets and slice centroids applied (an estimate when the
    positions are taken elsewhere in the ring)."""
    name = type(obj).__name__
    if x is None:
        x = y = np.zeros(1)
    if name == "Drift":
        return FLOPS_DRIFT
    if name == "DriftExact":
        return FLOPS_DRIFT_EXACT
    if name == "Multipole":
        return multipole_flops(int(obj.order), bool(obj.hxl != 0.0 or obj.hyl != 0.0))
    if name == "Cavity":
        return FLOPS_CAVITY
    if name == "XYShift":
        return FLOPS_XYSHIFT
    if name == "SRotation":
        return FLOPS_SROTATION
    if name == "LimitRect":
        return FLOPS_LIMIT_RECT
    if name == "LimitEllipse":
        return FLOPS_LIMIT_ELLIPSE
    if name == "LimitRectEllipse":
        return FLOPS_LIMIT_RECT_ELLIPSE
    if name == "DipoleEdge":
        return FLOPS_DIPEDGE
    if name == "TriCub":
        return FLOPS_TRICUB
    if name == "BeamBeam4D":
        d = np.asarray(obj.data)
        if d[10] <= 0.0:
            return 0
        return FLOPS_BB4D_BASE + _field_flops(x - d[6], y - d[7], d[2], d[3], d[5], False)
    if name == "SCQGaussProfile":
        if not int(obj.enabled):
            return 0
        base = FLOPS_SC_QGAUSS_BASE + (0 if abs(1.0 - obj.q_param) < 1e-6 else
                                       FLOPS_SC_QGAUSS_Q_NOT_1)
        return base + _field_flops(x - obj.x_co, y - obj.y_co, obj.sigma_x, obj.sigma_y,
                                   obj.min_sigma_diff, False)
    if name == "SCCoasting":
        if not int(obj.enabled):
            return 0
        return FLOPS_SC_COASTING_BASE + _field_flops(x - obj.x_co, y - obj.y_co, obj.sigma_x,
                                                     obj.sigma_y, obj.min_sigma_diff, False)
    if name == "BeamBeam6D":
        d = np.asarray(obj.data)
        if d[33] <= 0.0:
            return 0
        n = int(d.view(np.uint64)[18])
        s11, s13, s33 = d[6], d[8], d[13]
        singular = (s11 - s33) ** 2 + 4.0 * s13 * s13 < d[17]
        branch = FLOPS_BB6D_SINGULAR if singular else FLOPS_BB6D_REGULAR
        sx, sy = np.sqrt(s11), np.sqrt(s33)
        x0, y0 = x - d[21] - d[19], y - d[23] - d[20]
        xs, ys = d[38 + n:38 + 2 * n], d[38 + 2 * n:38 + 3 * n]
        fields = sum(_field_flops(x0 - xs[k], y0 - ys[k], sx, sy, d[16], True)
                     for k in range(n))
        return FLOPS_BB6D_ELEMENT + n * (FLOPS_BB6D_SLICE + branch) + fields
    return 0


def lattice_flops_per_pet(elements, x=None, y=None) -> float:
    """Average algorithmic FP64 operations per particle-element-turn of a
    lattice (Elements): element_flops averaged over its elements."""
    objs = list(elements.get_elements())
    if x is not None:
        x = np.asarray(x, dtype=np.float64)
        y = np.asarray(y, dtype=np.float64)
    return float(sum(element_flops(o, x, y) for o in objs)) / max(len(objs), 1)
