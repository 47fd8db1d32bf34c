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
        else:
            f = 0
        tot += f
        n += 1
    return tot / max(n, 1)
