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
