"""The Python particle-set API of the reference (python/sixtracklib/
particles.py) on the CPU: column keywords and defaults, derived quantities,
copies, differences and comparisons, pysixtrack transfers."""

from types import SimpleNamespace

import numpy as np
import pytest

from sixtracklib_gb300 import (ParticlesSet, calcParticlesDifference,
                               compareParticlesDifference, makeCopy)
from sixtracklib_gb300.particles import FIELDS, Particles


def test_defaults_and_keywords():
    p = Particles(num_particles=4)
    assert np.all(p.mass0 == Particles.pmass) and np.all(p.beta0 == 1.0)
    assert np.all(p.gamma0 == 1.0) and np.all(p.p0c == 1.0) and np.all(p.q0 == 0.0)
    assert np.all(p.rpp == 1.0) and np.all(p.rvv == 1.0) and np.all(p.state == 1)
    q = Particles(num_particles=3, x=[1e-3, 2e-3, 3e-3], p0c=7e12, at_element_id=5)
    np.testing.assert_array_equal(q.x, [1e-3, 2e-3, 3e-3])
    assert np.all(q.p0c == 7e12) and np.all(q.at_element == 5)
    with pytest.raises(TypeError):
        Particles(num_particles=2, xx=1.0)
    ps = ParticlesSet()
    r = ps.Particles(num_particles=2, zeta=[0.1, -0.1])
    np.testing.assert_array_equal(ps.particles[0].zeta, [0.1, -0.1])
    assert r.num_particles == 2


def test_derived_quantities():
    p = Particles.from_ref(num_particles=3, p0c=20e9)
    p.set_delta([0.0, 1e-3, -2e-3])
    b0 = p.beta0
    ptau = np.sqrt(p.delta ** 2 + 2 * p.delta + 1 / b0 ** 2) - 1 / b0
    np.testing.assert_allclose(p.ptau, ptau, rtol=1e-15)
    # ptau / beta0 = psigma: the set_delta of NS(Particles_update_delta_value)
    np.testing.assert_allclose(p.ptau / b0, p.psigma, rtol=1e-9, atol=1e-18)
    np.testing.assert_allclose(p.beta, b0 * p.rvv, rtol=1e-14)
    p.zeta[:] = 0.01
    np.testing.assert_allclose(p.sigma, 0.01 / p.rvv, rtol=1e-14)


def test_copy_difference_compare():
    p = Particles.from_ref(num_particles=5, p0c=7e12)
    p.x[:] = np.linspace(-1e-3, 1e-3, 5)
    c = makeCopy(p)
    for name in FIELDS:
        np.testing.assert_array_equal(getattr(c, name), getattr(p, name))
    assert compareParticlesDifference(p, c) == 0
    c.x[2] += 1e-12
    assert compareParticlesDifference(c, p) == +1 and compareParticlesDifference(p, c) == -1
    assert compareParticlesDifference(c, p, abs_treshold=1e-11) == 0
    d = calcParticlesDifference(c, p)
    assert d.x[2] == pytest.approx(1e-12) and np.count_nonzero(d.x) == 1
    c.x[2] = p.x[2]
    c.at_turn[4] = 3
    assert compareParticlesDifference(c, p, abs_treshold=1.0) == +1  # integers: exact
    c.at_turn[4] = 0
    c.x[0] = np.nan
    p.x[0] = np.nan
    assert compareParticlesDifference(c, p) == 0  # NaN neither greater nor smaller
    assert compareParticlesDifference(p, Particles(num_particles=4)) == -1
    assert compareParticlesDifference(Particles(), Particles()) == -1


def test_pysixtrack_transfer():
    p = Particles.from_ref(num_particles=2, p0c=7e12)
    p.set_delta([1e-4, -1e-4])
    p.x[:] = [1e-3, -1e-3]
    p.at_turn[1] = 7
    other = SimpleNamespace()
    p.to_pysixtrack(other, 1)
    assert other.x == -1e-3 and other.turn == 7 and other.qratio == 1.0
    assert other._update_coordinates is True and other.partid == 1
    q = Particles(num_particles=2)
    other.rpp, other.rvv = p.rpp[1], p.rvv[1]
    q.from_pysixtrack(other, 0)
    for name in FIELDS:
        if name != "particle_id":
            assert getattr(q, name)[0] == getattr(p, name)[1], name
    assert q.particle_id[0] == 1


def test_stcommon_q_gauss_helpers():
    """As the reference's tests/python/test_qgauss.py: for q = 1 the
    q-Gaussian is the normal density (rms sigma) to 1e-16; for q != 1 it
    integrates to 1 over its support."""
    from sixtracklib_gb300 import stcommon as sc

    for sigma in (1.0, 2.37):
        sb = sc.Math_sqrt_beta_from_gauss_sigma(sigma)
        xs = np.linspace(-4 * sigma, 4 * sigma, 101)
        ref = np.exp(-0.5 * (xs / sigma) ** 2) / np.sqrt(2 * np.pi * sigma * sigma)
        got = np.array([sc.Math_q_gauss(x, 1.0, sb) for x in xs])
        assert np.allclose(ref, got, 1e-16, 1e-16)
        shifted = np.array([sc.Math_q_gauss(x + 0.3, 1.0, sb, mu=0.3) for x in xs])
        np.testing.assert_allclose(shifted, got, rtol=1e-12)  # (x + 0.3) - 0.3 != x
    for q in (0.7, 1.3, 2.0):
        sb = 1.5
        lo = max(sc.Math_q_gauss_min_support(q, sb), -200.0)
        hi = min(sc.Math_q_gauss_max_support(q, sb), 200.0)
        xs = np.linspace(lo, hi, 400001)
        vals = np.array([sc.Math_q_gauss(x, q, sb) for x in xs[::50]])
        integral = np.trapezoid(vals, xs[::50])
        # q = 2 has 1 / x^2 tails: 2e-3 of it lies beyond +-200
        assert abs(integral - 1.0) < (5e-3 if q >= 2.0 else 1e-4), (q, integral)
    assert sc.st_ARCH_BEAM_ELEMENTS_BUFFER_ID.value == 2
    assert sc.st_ARCH_MIN_USER_DEFINED_BUFFER_ID.value == 1024
    assert sc.st_Buffer_new is not None and sc.st_NullBuffer is None
    with pytest.raises(AttributeError):
        sc.st_Not_a_function


def test_package_exports_the_reference_names():
    """The names python/sixtracklib/__init__.py exports for this path."""
    import sixtracklib_gb300 as st

    for name in ("Particles", "ParticlesSet", "ParticlesAddr", "makeCopy",
                 "calcParticlesDifference", "compareParticlesDifference", "Buffer",
                 "get_cbuffer_from_obj", "AssignAddressItem", "CudaTrackJob", "TrackJob",
                 "supports", "LineDensityProfileData",
                 "LineDensityProfileData_create_buffer_assignment", "TriCub", "TriCubData",
                 "TriCub_buffer_create_assign_address_item", "Elements", "Drift", "Multipole",
                 "BeamBeam6D", "SCQGaussProfile", "BeamMonitor"):
        assert hasattr(st, name), name
    assert st.supports("cuda") and not st.supports("opencl") and not st.supports("cpu")
