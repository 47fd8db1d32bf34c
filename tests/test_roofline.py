"""The frozen algorithmic FP64 operation counts (sixtracklib_gb300/roofline.py)
behind the bench line's roofline fractions."""

import numpy as np

from sixtracklib_gb300 import lattices, roofline


def test_plain_ring_counts_agree_between_the_two_entry_points():
    ring = lattices.synthetic_ring()
    assert roofline.lattice_flops_per_pet(ring) == roofline.lattice_flops_per_element(ring.cbuffer)
    assert abs(roofline.lattice_flops_per_element(ring.cbuffer) - 27.79) < 0.01


def test_cerrf_operation_count_follows_the_cern_regions():
    # outside the rectangle: 9 continued-fraction steps
    assert roofline.cerrf_flops(6.0, 1.0) == 9 * 11 + 2
    assert roofline.cerrf_flops(0.5, 5.0) == 9 * 11 + 2
    # at the origin: q = 1, nu = 31, nc = 30, plus exp(-x^2) for y == 0
    assert roofline.cerrf_flops(0.0, 0.0) == 14 + 31 * 11 + 30 * 8 + 2 + 2
    # y < 0 adds the reflection
    assert roofline.cerrf_flops(1.0, -1.0) == roofline.cerrf_flops(1.0, 1.0) + 20
    # the count falls towards the rectangle's edge
    f = roofline.cerrf_flops(np.linspace(0, 5.3, 50), np.zeros(50) + 0.1)
    assert np.all(np.diff(f) <= 0)


def test_beam_field_mix_counts():
    p = lattices.gaussian_particles(2048, seed=3)
    round_mix = roofline.lattice_flops_per_pet(lattices.bb_sc_ring(), p.x, p.y)
    ell_mix = roofline.lattice_flops_per_pet(lattices.bb_sc_ring(elliptic=True), p.x, p.y)
    # ~68 flop per particle-element-turn estimated for the round mix from the
    # reference's formulas; the elliptic mix is dominated by the Faddeeva
    # function of its 200 space-charge kicks
    assert 60 < round_mix < 80
    assert 400 < ell_mix < 700
    objs = lattices.bb_sc_ring().get_elements()
    bb6d = [o for o in objs if type(o).__name__ == "BeamBeam6D"][0]
    n = int(np.asarray(bb6d.data).view(np.uint64)[18])
    per_slice = (roofline.FLOPS_BB6D_SLICE + roofline.FLOPS_BB6D_SINGULAR +
                 roofline.FIELD_ROUND + roofline.G_ROUND)
    assert roofline.element_flops(bb6d, p.x, p.y) == roofline.FLOPS_BB6D_ELEMENT + n * per_slice


def test_tricub_count():
    ring = lattices.tricub_field_ring()
    n = len(ring)
    per_pet = roofline.lattice_flops_per_pet(ring)
    assert roofline.FLOPS_TRICUB == 381
    fodo = lattices.fodo_ring()
    expect = (roofline.lattice_flops_per_pet(fodo) * len(fodo) + 64 * 381) / n
    assert abs(per_pet - expect) < 1e-9
    assert abs(roofline.lattice_flops_per_element(ring.cbuffer) - per_pet) < 1e-9
