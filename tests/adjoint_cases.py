"""Lattices for the derivative tests."""

import numpy as np

from sixtracklib_gb300.beam_elements import Elements


def misc_ring(n_cells=24, seed=11):
    """A ring using every map that has an adjoint: Drift, DriftExact,
    Multipole with curvature and length (so the b1/a1 terms enter), skew
    and sextupole components, SRotation, XYShift, DipoleEdge, two cavities,
    LimitEllipse and LimitRectEllipse.  Learnable: quadrupole, skew
    quadrupole, dipole (knl[0], ksl[0] of the curved multipoles),
    sextupole strengths and both cavity voltages."""
    rng = np.random.default_rng(seed)
    e = Elements()
    params = []
    for c in range(n_cells):
        e.Drift(length=1.5)
        i = len(e)
        # weak bend: the dipole components cancel the curvature kick on momentum
        e.Multipole(knl=[1e-6, 0.05, float(rng.normal(0, 0.1))], ksl=[-5e-7, 1e-3],
                    hxl=1e-6, hyl=-5e-7, length=1.0)
        if c % 6 == 0:
            params += [(i, "knl", 0), (i, "ksl", 0), (i, "knl", 1), (i, "knl", 2),
                       (i, "ksl", 1)]
        e.DriftExact(length=1.5)
        ang = float(rng.normal(0, 1e-3))
        e.SRotation(cos_z=float(np.cos(ang)), sin_z=float(np.sin(ang)))
        e.XYShift(dx=float(rng.normal(0, 1e-5)), dy=float(rng.normal(0, 1e-5)))
        e.Drift(length=1.5)
        i = len(e)
        e.Multipole(knl=[0.0, -0.05])
        if c % 6 == 3:
            params.append((i, "knl", 1))
        e.DipoleEdge(r21=1e-3, r43=-1e-3)
        e.LimitEllipse(a=0.02, b=0.015)
        if c % 12 == 5:
            params.append((len(e), "voltage"))
            e.Cavity(voltage=3e6, frequency=400e6, lag=180.0)
    e.LimitRectEllipse(max_x=0.02, max_y=0.02, a=0.022, b=0.018)
    return e, params
