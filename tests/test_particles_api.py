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


def test_element_fields_are_buffer_views(oracle):
    """Assigning a field of an element that belongs to a lattice writes the
    lattice buffer in place (the reference's CObject fields are views), so
    the edit reaches tracking; an array keeps its length."""
    import pytest

    from sixtracklib_gb300 import lattices

    e = lattices.fodo_ring()
    img0 = e.cbuffer.to_image().copy()
    d = e.get(0)
    d.length = 2.5
    assert e.get(0).length == 2.5
    assert np.count_nonzero(e.cbuffer.to_image() != img0) == 1
    m = e.get(1)
    m.bal = np.array([0.0, 0.0, 0.06, 0.0])
    assert np.allclose(e.get(1).bal, [0.0, 0.0, 0.06, 0.0])
    with pytest.raises(ValueError):
        m.bal = np.zeros(6)
    fresh = lattices.fodo_ring()
    fresh.get(0).length, fresh.get(1).bal = 2.5, np.array([0.0, 0.0, 0.06, 0.0])
    p = lattices.gaussian_particles(32, seed=1).block
    a, b = p.copy(), p.copy()
    oracle.track_until(e.cbuffer.to_image(), a, 2)
    oracle.track_until(fresh.cbuffer.to_image(), b, 2)
    assert np.array_equal(a, b)


def test_reference_element_helpers():
    """SRotation.angle (radians), the half-axes setters, the output monitors
    helper (beam_elements.py:293-299, 314-367, 460-467) and the
    ParticlesAddr buffer object (particles.py:490-513)."""
    import pytest

    from sixtracklib_gb300.beam_elements import (Elements, LimitEllipse,
                                                 append_beam_monitors_to_lattice)
    from sixtracklib_gb300.particles import ParticlesAddr, ParticlesSet

    e = Elements()
    r = e.SRotation(angle=30.0)
    assert abs(r.angle - np.pi / 6) < 1e-15 and abs(r.angle_deg - 30.0) < 1e-12
    el = e.LimitEllipse(a=0.02, b=0.01)
    el.set_half_axes(0.03, 0.015)
    got = e.get(1)
    assert (got.a_squ, got.b_squ, got.a_b_squ) == (0.03 * 0.03, 0.015 * 0.015,
                                                   (0.03 * 0.03) * (0.015 * 0.015))
    rel = e.LimitRectEllipse(max_x=0.02, max_y=0.02, a=0.02, b=0.02).set_half_axes_squ(4e-4, 1e-4)
    assert e.get(2).a_b_squ == 4e-4 * 1e-4 and rel.b_squ == 1e-4
    assert isinstance(LimitEllipse(a=1.0, b=2.0).set_half_axes(2.0, 3.0), LimitEllipse)
    n0 = len(e)
    assert append_beam_monitors_to_lattice(e, 2, 10, 107, skip_turns=10, max_particle_id=99) == 2
    tbt, out = e.get(n0), e.get(n0 + 1)
    assert (tbt.start, tbt.num_stores, tbt.skip, tbt.is_rolling) == (2, 8, 1, 0)
    assert (out.start, out.num_stores, out.skip, out.is_rolling) == (10, 10, 10, 1)
    assert out.max_particle_id == 99
    assert append_beam_monitors_to_lattice(e, 0, 0, 0) == 0
    ps = ParticlesSet()
    a = ParticlesAddr(cbuffer=ps.cbuffer, num_particles=4, x=4096)
    assert ps.cbuffer.objects[0].typeid == 512 and a.x == 4096
    with pytest.raises(ImportError):  # needs sixtracktools and pysixtrack, as the reference
        ParticlesSet.fromSixDump101("input", "dump.dat")
