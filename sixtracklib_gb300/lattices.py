"""Seeded synthetic lattices and particle distributions.

These generate the workloads the engine is measured and checked on.  All are
synthetic (no public dataset is involved) and fully determined by the seed:

* :func:`fodo_ring` -- 64 FODO cells (drift 2 m, focusing / defocusing quad
  kicks k1l = +-0.05), one 6 MV / 400 MHz cavity at lag 180 deg and one
  +-0.02 m LimitRect (258 elements);
* :func:`synthetic_ring` -- 20,000 elements: 9,000 drifts L~U(0.5,5) m,
  8,000 multipoles of order U{1..10} (k1l = +-U(0.01,0.05) alternating,
  b_n ~ N(0, 1e-4 * 10^-n)), 1,000 XYShift N(0,1e-5) m, 1,000 SRotation
  N(0,1e-4) rad, 16 cavities, 984 LimitEllipse (a=0.015, b=0.01);
* :func:`bb_sc_ring` -- the FODO ring plus 4 BeamBeam6D (21 slices), 4
  BeamBeam4D and 200 q-Gaussian space-charge kicks;
* :func:`sc_interpolated_ring` -- the FODO ring plus interpolated
  space-charge kicks on tabulated line densities;
* :func:`learnable_fodo_ring` -- the FODO ring with 64 quadrupole and 16
  sextupole strengths marked as learnable (differentiable tracking);
* :func:`tricub_field_ring` -- the FODO ring plus 64 TriCub kicks sharing one
  100 x 100 x 50 field map (a Gaussian potential bump);
* :func:`variant_ring` / :func:`batch_specs` -- rings built like the
  synthetic ring at any size, and the 256-variant batched workload;
* particle sets: Gaussian 6D and the polar amplitude grid.
"""

from __future__ import annotations

import numpy as np

from .beam_elements import (
    QELEM, BeamBeam4D, BeamBeam6D, Cavity, Drift, Elements, LimitEllipse,
    LimitRect, Multipole, SCQGaussProfile, SRotation, XYShift, bb6d_data,
)
from .particles import PROTON_MASS_EV, Particles

P0C = 7e12


def fodo_cells(elements: Elements, n_cells=64, k1l=0.05, drift=2.0):
    for _ in range(n_cells):
        elements.Drift(length=drift)
        elements.Multipole(knl=[0.0, +k1l])
        elements.Drift(length=drift)
        elements.Multipole(knl=[0.0, -k1l])


def fodo_ring(n_cells=64, with_cavity=True, with_aperture=True) -> Elements:
    """The plain FODO ring (258 elements)."""
    e = Elements()
    fodo_cells(e, n_cells)
    if with_cavity:
        e.Cavity(voltage=6e6, frequency=400e6, lag=180.0)
    if with_aperture:
        e.LimitRect(min_x=-0.02, max_x=0.02, min_y=-0.02, max_y=0.02)
    return e


def learnable_fodo_ring(seed=4, n_cells=64, n_sextupoles=16, k2l_sigma=0.1):
    """The FODO ring with learnable strengths: the 64 focusing quadrupoles'
    knl[1] and, on 16 of them (evenly spaced), a sextupole component knl[2]
    ~ N(0, 0.1).  Returns ``(elements, params)`` with ``params`` in the form
    :class:`sixtracklib_gb300.autodiff.DifferentiableLattice` takes: 64
    ``(element, "knl", 1)`` then 16 ``(element, "knl", 2)``."""
    rng = np.random.default_rng(seed)
    e = Elements()
    sext_cells = set(np.linspace(0, n_cells, n_sextupoles, endpoint=False).astype(int).tolist())
    quads, sexts = [], []
    for c in range(n_cells):
        e.Drift(length=2.0)
        if c in sext_cells:
            sexts.append(len(e))
            e.Multipole(knl=[0.0, +0.05, float(rng.normal(0.0, k2l_sigma))])
        else:
            e.Multipole(knl=[0.0, +0.05])
        quads.append(len(e) - 1)
        e.Drift(length=2.0)
        e.Multipole(knl=[0.0, -0.05])
    e.Cavity(voltage=6e6, frequency=400e6, lag=180.0)
    e.LimitRect(min_x=-0.02, max_x=0.02, min_y=-0.02, max_y=0.02)
    params = [(q, "knl", 1) for q in quads] + [(s, "knl", 2) for s in sexts]
    return e, params


def synthetic_ring(seed=20240601, n_cells=4000, n_extra_drift=1000,
                   n_shift=1000, n_rot=1000, n_cav=16, n_ell=984) -> Elements:
    """The 20,000-element synthetic ring.

    Linear structure: ``n_cells`` FODO cells [Drift L, QF +k, Drift L, QD -k]
    with L ~ U(0.5, 5) m per cell and k ~ U(0.01, 0.05).  The drawn k values
    are arranged as a slow ramp up and back down around the ring so that
    neighbouring cells are nearly matched; randomly ordered quad strengths
    make the one-turn map unstable (every particle is lost), this ordering
    keeps it stable.  Each multipole has order ~ U{1..10} with
    b_n ~ N(0, 1e-4 * 10^-n) for n >= 2.  ``n_extra_drift`` of the cell drifts
    (with L >= 1 m) are split in two halves; XYShift N(0,1e-5) m, SRotation
    N(0,1e-4) rad and LimitEllipse (a=0.015, b=0.01 m) are inserted after
    randomly chosen quads, the cavities (lag 180 deg) evenly around the ring.
    """
    rng = np.random.default_rng(seed)
    k = np.sort(rng.uniform(0.01, 0.05, n_cells))
    k = np.concatenate([k[0::2], k[1::2][::-1]])
    L = rng.uniform(0.5, 5.0, n_cells)
    orders = rng.integers(1, 11, size=2 * n_cells)
    split = np.zeros(2 * n_cells, dtype=bool)
    cand = np.nonzero(np.repeat(L, 2) >= 1.0)[0]
    split[rng.choice(cand, size=n_extra_drift, replace=False)] = True
    extras = {}
    kinds = [2] * n_shift + [3] * n_rot + [5] * n_ell
    slots = rng.choice(2 * n_cells, size=len(kinds), replace=True)
    for s_, kd in zip(slots, kinds):
        extras.setdefault(int(s_), []).append(kd)
    cav_slots = set(int(i) for i in np.linspace(0, 2 * n_cells, n_cav, endpoint=False))
    e = Elements()
    for c in range(n_cells):
        for h in range(2):
            j = 2 * c + h
            if split[j]:
                e.Drift(length=float(L[c] * 0.5))
                e.Drift(length=float(L[c] * 0.5))
            else:
                e.Drift(length=float(L[c]))
            order = int(orders[j])
            knl = np.zeros(order + 1)
            knl[1] = k[c] if h == 0 else -k[c]
            for n in range(2, order + 1):
                knl[n] = float(rng.normal(0.0, 1e-4 * 10.0 ** (-n)))
            e.Multipole(knl=list(knl))
            if j in cav_slots:
                e.Cavity(voltage=6e6 / n_cav, frequency=400e6, lag=180.0)
            for kd in extras.get(j, ()):
                if kd == 2:
                    e.XYShift(dx=float(rng.normal(0, 1e-5)), dy=float(rng.normal(0, 1e-5)))
                elif kd == 3:
                    ang = float(rng.normal(0.0, 1e-4))
                    e.SRotation(cos_z=float(np.cos(ang)), sin_z=float(np.sin(ang)))
                else:
                    e.LimitEllipse(a=0.015, b=0.01)
    return e


def sc_interpolated_ring(n_kicks=8, seed=3):
    """The FODO ring plus interpolated space-charge kicks: tabulated
    Gaussian line densities (linear and cubic interpolation, one table with
    interpolation switched off) and kicks without a table (fallback
    density).  Returns ``(elements, tables)``; ``tables`` (a
    :class:`~sixtracklib_gb300.sc_line_density.LineDensityBuffer`) owns the
    tables the kicks address and must stay alive while the lattice is
    compiled or tracked on the CPU."""
    from .sc_line_density import LineDensityBuffer

    rng = np.random.default_rng(seed)
    tables = LineDensityBuffer()
    z = np.linspace(-0.3, 0.3, 41)
    prof = np.exp(-0.5 * (z / 0.1) ** 2) * 1e12
    idx = [tables.add(prof, z0=-0.3, dz=float(z[1] - z[0]), method="linear", capacity=48),
           tables.add(prof * 1.1, z0=-0.3, dz=float(z[1] - z[0]), method="cubic"),
           tables.add(prof, z0=-0.3, dz=float(z[1] - z[0]), method="none")]
    e = fodo_ring()
    for k in range(n_kicks):
        which = k % 4
        addr = tables.address(idx[which]) if which < 3 else 0
        e.SCInterpolatedProfile(number_of_particles=1e11, length=0.5,
                                sigma_x=1e-3, sigma_y=float(rng.choice([1e-3, 1.2e-3])),
                                interpol_data_addr=addr, line_density_prof_fallback=5e11,
                                min_sigma_diff=1e-10)
    return e, tables


def gaussian_bump_table(nx, ny, nz, dx, dy, dz, x0, y0, z0, amplitude, sx, sy, sz):
    """Node table of phi = amplitude exp(-x^2/2sx^2 - y^2/2sy^2 - z^2/2sz^2)
    for a TriCubData: f, f_x, f_y, f_z, f_xy, f_xz, f_yz, f_xyz at every
    node, the derivatives scaled by the grid steps, at l + 8 (ix + nx (iy +
    ny iz))."""
    def axis(n, d, o, s):
        u = o + d * np.arange(n)
        g = np.exp(-0.5 * (u / s) ** 2)
        return g, -u / (s * s) * g * d  # value, derivative times the step

    gx, dgx = axis(nx, dx, x0, sx)
    gy, dgy = axis(ny, dy, y0, sy)
    gz, dgz = axis(nz, dz, z0, sz)
    kinds = [(gx, gy, gz), (dgx, gy, gz), (gx, dgy, gz), (gx, gy, dgz),
             (dgx, dgy, gz), (dgx, gy, dgz), (gx, dgy, dgz), (dgx, dgy, dgz)]
    t = np.empty((nz, ny, nx, 8))
    for l, (a, b, c) in enumerate(kinds):
        t[..., l] = amplitude * c[:, None, None] * b[None, :, None] * a[None, None, :]
    return t.reshape(-1)


def tricub_field_ring(n_kicks=64, length=0.5, amplitude=2e-11) -> Elements:
    """The FODO ring plus ``n_kicks`` TriCub kicks (spread over the ring's
    cells) that share one TriCubData: a 100 x 100 x 50 grid over +-12.4 mm
    transversely and +-0.49 m longitudinally holding a Gaussian potential
    bump (sigma 3 mm x 2.5 mm x 0.2 m); kicks of order 1e-8 rad.  The
    TriCubData is the last element (skipped when the map is enabled)."""
    e = fodo_ring()
    n_fodo = len(e)
    out = Elements()
    step = max(1, n_fodo // n_kicks)
    data_index = n_fodo + n_kicks
    k = 0
    for i, o in enumerate(e.get_elements()):
        out.cbuffer.add_raw(e.cbuffer.objects[i])
        if k < n_kicks and i % step == step - 1:
            out.TriCub(data=data_index, length=length)
            k += 1
    while k < n_kicks:
        out.TriCub(data=data_index, length=length)
        k += 1
    nx, ny, nz = 100, 100, 50
    dx = dy = 0.25e-3
    dz = 0.02
    x0, y0, z0 = -0.5 * (nx - 1) * dx, -0.5 * (ny - 1) * dy, -0.5 * (nz - 1) * dz
    out.TriCubData(nx=nx, ny=ny, nz=nz, x0=x0, y0=y0, z0=z0, dx=dx, dy=dy, dz=dz,
                   table_addr=gaussian_bump_table(nx, ny, nz, dx, dy, dz, x0, y0, z0,
                                                  amplitude, 3e-3, 2.5e-3, 0.2))
    return out


def variant_ring(seed: int, n_elements: int) -> Elements:
    """A ring built like :func:`synthetic_ring`, scaled to about
    ``n_elements`` elements (cells, split drifts, shifts, rotations,
    apertures and cavities in the same proportions), with its own seeded
    quadrupole ramp and multipole errors."""
    f = max(n_elements, 100) / 20000.0
    n_cells = max(4, int(round(4000 * f)))
    n_extra = min(int(round(1000 * f)), n_cells)  # at most one split per cell pair
    return synthetic_ring(seed=seed, n_cells=n_cells, n_extra_drift=n_extra,
                          n_shift=int(round(1000 * f)), n_rot=int(round(1000 * f)),
                          n_cav=max(1, int(round(16 * f))), n_ell=int(round(984 * f)))


def batch_specs(n_variants=256, seed=2025, elements=(500, 20000), particles=(1024, 262144)):
    """The batched-tracking workload: per variant ``(lattice seed, element
    count ~ U(elements), particle count ~ log-uniform(particles), particle
    seed)``."""
    rng = np.random.default_rng(seed)
    e = rng.uniform(elements[0], elements[1], n_variants).astype(int)
    n = np.exp(rng.uniform(np.log(particles[0]), np.log(particles[1]), n_variants)).astype(int)
    return [(int(seed * 1000 + v), int(e[v]), int(n[v]), int(seed * 7919 + v))
            for v in range(n_variants)]


def bb_sc_ring(seed=7, n_bb6d=4, n_bb4d=4, n_sc=200, n_slices=21,
               sigma_x=16.7e-6, sigma_y=16.7e-6, sigma_z=0.0755,
               bunch_charge=1.15e11, elliptic=False) -> Elements:
    """FODO ring plus beam-beam and space-charge kicks (BB6D uses a Gaussian
    longitudinal slicing of the strong bunch into equal-charge slices)."""
    rng = np.random.default_rng(seed)
    e = fodo_ring()
    sx, sy = sigma_x, (sigma_y * 1.3 if elliptic else sigma_y)
    # equal-charge Gaussian slice centroids
    from math import erf, sqrt

    edges = np.linspace(0, 1, n_slices + 1)
    z = np.zeros(n_slices)
    for i in range(n_slices):
        mid = 0.5 * (edges[i] + edges[i + 1])
        lo, hi = -8.0, 8.0
        for _ in range(80):
            m = 0.5 * (lo + hi)
            if 0.5 * (1 + erf(m / sqrt(2))) < mid:
                lo = m
            else:
                hi = m
        z[i] = 0.5 * (lo + hi) * sigma_z
    n_per_slice = np.full(n_slices, bunch_charge / n_slices)
    for i in range(n_bb6d):
        data = bb6d_data(
            q_part=QELEM, phi=float(rng.uniform(1e-4, 2e-4)), alpha=float(rng.uniform(0, 0.5)),
            delta_x=float(rng.normal(0, 1e-6)), delta_y=float(rng.normal(0, 1e-6)),
            n_part_per_slice=n_per_slice, z_slices=z,
            sigmas=(sx * sx, 0.0, 0.0, 0.0, 1e-12, 0.0, 0.0, sy * sy, 0.0, 1e-12),
            min_sigma_diff=1e-10, threshold_singular=1e-28)
        e.BeamBeam6D(data=data)
        e.Drift(length=1.0)
    for i in range(n_bb4d):
        e.BeamBeam4D(charge=bunch_charge, sigma_x=sx, sigma_y=sy, beta_r=1.0,
                     min_sigma_diff=1e-10, x_bb=float(rng.normal(0, 1e-6)),
                     y_bb=float(rng.normal(0, 1e-6)), d_px=0.0, d_py=0.0, enabled=1.0)
        e.Drift(length=1.0)
    for i in range(n_sc):
        e.SCQGaussProfile(number_of_particles=1e11, bunchlength_rms=0.1,
                          sigma_x=1e-3, sigma_y=(1.2e-3 if elliptic else 1e-3),
                          length=0.1, x_co=0.0, y_co=0.0, min_sigma_diff=1e-10,
                          q_param=1.0, enabled=1)
    return e


def gaussian_particles(n, seed=12345, sx=1e-3, spx=1e-5, sy=1e-3, spy=1e-5,
                       sz=0.05, sdelta=1e-4, p0c=P0C) -> Particles:
    rng = np.random.default_rng(seed)
    p = Particles(num_particles=n).set_reference(p0c=p0c, mass0=PROTON_MASS_EV, q0=1.0)
    p.x[:] = rng.normal(0, sx, n)
    p.px[:] = rng.normal(0, spx, n)
    p.y[:] = rng.normal(0, sy, n)
    p.py[:] = rng.normal(0, spy, n)
    p.zeta[:] = rng.normal(0, sz, n)
    p.set_delta(rng.normal(0, sdelta, n))
    return p


def polar_grid_particles(n=1_000_000, n_angles=11, max_sigma=20.0, sigma=1e-3,
                         seed=99, p0c=P0C) -> Particles:
    """Polar amplitude grid: ceil(n/11) radii in [0, 20 sigma] x 11 angles,
    truncated to n; delta ~ U(-3e-4, 3e-4)."""
    rng = np.random.default_rng(seed)
    n_r = -(-n // n_angles)
    r = np.linspace(0.0, max_sigma * sigma, n_r)
    th = np.linspace(0.0, 0.5 * np.pi, n_angles)
    rr, tt = np.meshgrid(r, th, indexing="ij")
    x = (rr * np.cos(tt)).reshape(-1)[:n]
    y = (rr * np.sin(tt)).reshape(-1)[:n]
    p = Particles(num_particles=n).set_reference(p0c=p0c, mass0=PROTON_MASS_EV, q0=1.0)
    p.x[:] = x
    p.y[:] = y
    p.set_delta(rng.uniform(-3e-4, 3e-4, n))
    return p
