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


def field_ring(seed=5):
    """The FODO ring with every thin field kick that has an adjoint: 4D
    beam-beam (round and elliptic strong beams), coasting space charge (round
    and elliptic), q-Gaussian space charge (q = 1, 1.2, 0.8), interpolated
    space charge (linear, cubic, fallback) and an RF multipole.  Learnable:
    two quadrupole strengths and the cavity voltage.  Returns
    ``(elements, params, tables)``; ``tables`` owns the line-density tables
    and must stay alive while the lattice is compiled or tracked."""
    from sixtracklib_gb300 import lattices
    from sixtracklib_gb300.beam_elements import QELEM
    from sixtracklib_gb300.sc_line_density import LineDensityBuffer

    rng = np.random.default_rng(seed)
    e = lattices.fodo_ring()
    params = [(1, "knl", 1), (3, "knl", 1), (256, "voltage")]
    tables = LineDensityBuffer()
    z = np.linspace(-0.3, 0.3, 41)
    prof = np.exp(-0.5 * (z / 0.1) ** 2) * 1e12
    t_lin = tables.add(prof, z0=-0.3, dz=float(z[1] - z[0]), method="linear", capacity=48)
    t_cub = tables.add(prof, z0=-0.3, dz=float(z[1] - z[0]), method="cubic", capacity=44)
    for sx, sy in ((2e-3, 2e-3), (2e-3, 1.5e-3), (1.4e-3, 2.2e-3)):
        e.BeamBeam4D(charge=2e10, sigma_x=sx, sigma_y=sy, beta_r=1.0, min_sigma_diff=1e-10,
                     x_bb=float(rng.normal(0, 1e-4)), y_bb=float(rng.normal(0, 1e-4)),
                     d_px=1e-9, d_py=-1e-9, enabled=1.0)
        e.Drift(length=0.5)
    for sx, sy in ((1e-3, 1e-3), (1e-3, 1.3e-3)):
        e.SCCoasting(number_of_particles=5e11, circumference=500.0, sigma_x=sx, sigma_y=sy,
                     length=1.0, x_co=1e-5, y_co=-1e-5, min_sigma_diff=1e-10)
    for q in (1.0, 1.2, 0.8):
        e.SCQGaussProfile(number_of_particles=1e11, bunchlength_rms=0.1, sigma_x=1e-3,
                          sigma_y=1.2e-3, length=0.5, x_co=0.0, y_co=0.0, min_sigma_diff=1e-10,
                          q_param=q, enabled=1)
    # the kick scales with number_of_particles x line density
    # (be_beamfields/track.h:291-315): the tables carry the density
    for addr in (tables.address(t_lin), tables.address(t_cub), 0):
        e.SCInterpolatedProfile(number_of_particles=1.0, length=0.5, sigma_x=1.1e-3,
                                sigma_y=1e-3, interpol_data_addr=addr,
                                line_density_prof_fallback=5e11, min_sigma_diff=1e-10)
    e.RFMultipole(voltage=1e5, frequency=400e6, lag=30.0, knl=[1e-6, 1e-3, 0.05],
                  ksl=[0.0, 2e-4], pn=[10.0, 20.0, 0.0], ps=[5.0, 0.0])
    assert isinstance(QELEM, float)
    return e, params, tables


def bb6d_ring(p0c, n_slices=5, sigma_z=0.08):
    """The FODO ring with three 6D beam-beam elements, one per branch of the
    strong beam's sigma-matrix propagation and field: a round uncoupled beam
    (singular branch, round field, crossing angle 1 mrad), a coupled
    elliptic beam (general branch, sigma_x > sigma_y, 2 mrad in a tilted
    plane) and an uncoupled elliptic beam with sigma_x < sigma_y (head on);
    closed orbit, separation and dipolar subtraction are non-zero.  The
    strong bunch, 1e10 x p0c / 20 GeV protons in equal-charge slices, gives
    a beam-beam parameter of a few 1e-3 at any energy.  Learnable: two
    quadrupole strengths and the cavity voltage."""
    from math import erf, sqrt

    from sixtracklib_gb300 import lattices
    from sixtracklib_gb300.beam_elements import QELEM, bb6d_data

    rng = np.random.default_rng(17)
    e = lattices.fodo_ring()
    params = [(1, "knl", 1), (3, "knl", 1), (256, "voltage")]
    edges = np.linspace(0.0, 1.0, n_slices + 1)
    z = np.zeros(n_slices)
    for i in range(n_slices):  # Gaussian quantile of each slice's middle
        lo, hi, mid = -8.0, 8.0, 0.5 * (edges[i] + edges[i + 1])
        for _ in range(80):
            m = 0.5 * (lo + hi)
            lo, hi = (m, hi) if 0.5 * (1 + erf(m / sqrt(2))) < mid else (lo, m)
        z[i] = 0.5 * (lo + hi) * sigma_z
    n_part = np.full(n_slices, 1e10 * p0c / 20e9 / n_slices)
    A = np.diag([1e-3, 2e-3, 1e-3, 2e-3]) @ (np.eye(4) + 0.3 * rng.normal(size=(4, 4)))
    sig = A @ A.T
    coupled = [sig[i, j] for i, j in ((0, 0), (0, 1), (0, 2), (0, 3), (1, 1), (1, 2), (1, 3),
                                      (2, 2), (2, 3), (3, 3))]
    beams = [((1e-6, 0, 0, 0, 4e-6, 0, 0, 1e-6, 0, 4e-6), 1e-3, 0.2),
             (tuple(coupled), 2e-3, 1.0),
             ((0.7e-6, 0.2e-6, 0, 0, 2e-6, 0, 0, 1.3e-6, -0.3e-6, 5e-6), 0.0, 0.0)]
    for sigmas, phi, alpha in beams:
        e.BeamBeam6D(data=bb6d_data(
            q_part=QELEM, phi=phi, alpha=alpha, delta_x=float(rng.normal(0, 1e-4)),
            delta_y=float(rng.normal(0, 1e-4)), n_part_per_slice=n_part, z_slices=z,
            sigmas=sigmas, co=(1e-5, 1e-7, -1e-5, 2e-7, 1e-3, 1e-6),
            d_sub=(1e-6, 1e-8, -1e-6, 2e-8, 1e-4, 1e-7)))
        e.Drift(length=0.5)
    return e, params
