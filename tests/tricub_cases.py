"""Lattices for the TriCub map and the map feature flags (tests and
tests/golden/make_golden.py).

* ``kicks_case``: the reference's TriCub known-answer test
  (tests/python/beam_elements/test_tricub.py:9-113): a 5 x 7 x 9 grid of
  uniform random values (numpy's legacy generator seeded with the seed
  stored beside the kicks, tests/testdata/tricub/precomputed_kicks.txt),
  derivatives scaled by the grid steps, one TriCub of length 1 and 1,000
  particles inside the grid, one turn; the expected px, py, ptau are the
  stored kicks.
* ``tricub_ring``: the FODO ring with two TriCub kicks (one mirrored in x
  and z, one shifted with dipolar kick corrections) on grids that hold the
  whole beam for the turns tracked, so the reference never reads outside
  its table.
* ``flags_lattice``: one element of every type a feature flag governs
  (TriCub and its data, BeamBeam4D, BeamBeam6D, SCCoasting,
  SCQGaussProfile, SCInterpolatedProfile) between drifts.
"""

from __future__ import annotations

import numpy as np

from sixtracklib_gb300 import lattices
from sixtracklib_gb300.beam_elements import Elements, bb6d_data
from sixtracklib_gb300.particles import Particles

# test_tricub.py:48-56
KICKS_GRID = dict(nx=5, ny=7, nz=9, dx=0.001, dy=0.002, dz=0.003)


def scaled_table(values: np.ndarray, dx: float, dy: float, dz: float) -> np.ndarray:
    """The node table of values[ix, iy, iz, l] with the derivatives scaled
    by the grid steps (scale order of test_tricub.py:85), laid out at
    l + 8 (ix + nx (iy + ny iz))."""
    scale = np.array([1.0, dx, dy, dz, dx * dy, dx * dz, dy * dz, (dx * dy) * dz])
    t = values * scale  # [ix, iy, iz, l]
    return np.ascontiguousarray(t.transpose(2, 1, 0, 3)).reshape(-1)


def kicks_case(seed: int, n_part: int = 1000):
    """(elements, particles) of the reference's known-answer test."""
    g = KICKS_GRID
    nx, ny, nz, dx, dy, dz = g["nx"], g["ny"], g["nz"], g["dx"], g["dy"], g["dz"]
    rs = np.random.RandomState(seed)
    values = rs.rand(nx, ny, nz, 8) * 1.0e-3
    x0, y0, z0 = -(nx // 2) * dx, -(ny // 2) * dy, -(nz // 2) * dz
    tx = x0 + (nx - 2) * dx * rs.rand(n_part)
    ty = y0 + (ny - 2) * dy * rs.rand(n_part)
    tz = z0 + (nz - 2) * dz * rs.rand(n_part)
    e = Elements()
    e.TriCub(data=1, length=1.0)
    e.TriCubData(nx=nx, ny=ny, nz=nz, x0=x0, y0=y0, z0=z0, dx=dx, dy=dy, dz=dz,
                 table_addr=scaled_table(values, dx, dy, dz))
    # pysixtrack's default particle (1 GeV/c protons), tau = test_z
    p = Particles.from_ref(num_particles=n_part, p0c=1e9)
    p.x[:] = tx
    p.y[:] = ty
    p.zeta[:] = p.beta0 * tz
    p.particle_id[:] = np.arange(n_part)
    return e, p


def _grid(e: Elements, rng, nx, ny, nz, dx, dy, dz, x0, y0, z0, mirror=(0, 0, 0),
          scale=1e-9):
    values = rng.uniform(-1.0, 1.0, (nx, ny, nz, 8)) * scale
    e.TriCubData(nx=nx, ny=ny, nz=nz, x0=x0, y0=y0, z0=z0, dx=dx, dy=dy, dz=dz,
                 mirror_x=mirror[0], mirror_y=mirror[1], mirror_z=mirror[2],
                 table_addr=scaled_table(values, dx, dy, dz))
    return len(e) - 1


def tricub_ring(seed: int = 5) -> Elements:
    """FODO ring + TriCub A (mirrored in x and z, grid from 0) + TriCub B
    (shifted, with dipolar kick corrections) + their two TriCubData."""
    rng = np.random.default_rng(seed)
    e = lattices.fodo_ring()
    n = len(e)
    # data objects after the two kicks: indices n + 2 and n + 3
    e.TriCub(data=n + 2, length=0.8, x_shift=0.0, y_shift=0.0, tau_shift=0.0)
    e.TriCub(data=n + 3, length=1.2, x_shift=2e-4, y_shift=-1e-4, tau_shift=0.01,
             dipolar_kick_px=3e-10, dipolar_kick_py=-2e-10, dipolar_kick_ptau=1e-11)
    _grid(e, rng, 13, 11, 9, 2e-3, 2e-3, 0.1, 0.0, -10e-3, 0.0, mirror=(1, 0, 1))
    _grid(e, rng, 14, 12, 10, 2e-3, 2e-3, 0.09, -13e-3, -11e-3, -0.4)
    return e


def tricub_particles(n: int, seed: int) -> Particles:
    return lattices.gaussian_particles(n, seed=seed, sx=1e-3, sy=1e-3, sz=0.05)


def flags_lattice(seed: int = 3) -> Elements:
    """TriCub (+ data), BeamBeam4D, BeamBeam6D, SCCoasting, SCQGaussProfile
    and SCInterpolatedProfile (fallback density) between drifts."""
    rng = np.random.default_rng(seed)
    e = Elements()
    e.Drift(length=0.5)
    e.TriCub(data=2, length=1.0)
    _grid(e, rng, 13, 13, 9, 2e-3, 2e-3, 0.1, -12e-3, -12e-3, -0.4)
    e.Drift(length=0.5)
    e.BeamBeam4D(charge=1.15e11, sigma_x=1e-3, sigma_y=1.2e-3, beta_r=1.0,
                 min_sigma_diff=1e-10, x_bb=1e-5, y_bb=-1e-5, d_px=0.0, d_py=0.0, enabled=1.0)
    e.Drift(length=0.5)
    z = np.array([-0.05, 0.0, 0.05])
    e.BeamBeam6D(data=bb6d_data(
        q_part=1.602176634e-19, phi=1.5e-4, alpha=0.3, delta_x=1e-6, delta_y=-1e-6,
        n_part_per_slice=np.full(3, 1.15e11 / 3), z_slices=z,
        sigmas=(1e-6, 0.0, 0.0, 0.0, 1e-12, 0.0, 0.0, 1.2e-6, 0.0, 1e-12),
        min_sigma_diff=1e-10, threshold_singular=1e-28))
    e.Drift(length=0.5)
    e.SCCoasting(number_of_particles=1e11, circumference=1000.0, sigma_x=1e-3,
                 sigma_y=1.5e-3, length=1.0)
    e.Drift(length=0.5)
    e.SCQGaussProfile(number_of_particles=1e11, bunchlength_rms=0.1, sigma_x=1e-3,
                      sigma_y=1.2e-3, length=0.5, q_param=1.0, min_sigma_diff=1e-10)
    e.Drift(length=0.5)
    e.SCInterpolatedProfile(number_of_particles=1e11, length=0.5, sigma_x=1e-3,
                            sigma_y=1e-3, interpol_data_addr=0,
                            line_density_prof_fallback=5e11, min_sigma_diff=1e-10)
    e.Drift(length=0.5)
    return e


# (bb4d, bb6d, spacecharge, tricub) per reference build, 2 enabled, 1 skip,
# 0 disabled: the default build and the two of oracle/build_ref.sh
FLAG_BUILDS = {"default": (2, 2, 2, 0), "a": (1, 0, 1, 2), "b": (0, 1, 0, 1)}
_WORDS = {2: "enabled", 1: "skip", 0: "disabled"}


def flags_config(flags) -> str:
    """The engine's configuration keys for a flag tuple."""
    bb4d, bb6d, sc, tc = flags
    return (f"track_beambeam4d={_WORDS[bb4d]} track_beambeam6d={_WORDS[bb6d]} "
            f"track_spacecharge={_WORDS[sc]} track_tricub={_WORDS[tc]}")
