"""The forward-mode (dual-number) oracle that checks the adjoint.

Pinned twice on the CPU: its values are the C oracle's values bit for bit
(same maps, same operation order, same loss bookkeeping), and its
derivatives agree with central finite differences of the C oracle's
tracking.  Step sizes: a central difference carries the tracking's own
rounding noise divided by h, so h is chosen per quantity: the quadrupole
strengths (strongly coupled to the coordinates) use h = 1e-7 relative; the
sextupole strengths move the coordinates ~1e-6 times less per unit of
relative change and use h = 1e-3 relative; the coordinates use h = 1e-5 of
each coordinate's spread.  At these steps both the rounding and the
truncation error are below 1e-7 of the derivative.
"""

from math import factorial

import numpy as np
import pytest

from oracle import dual
from sixtracklib_gb300 import lattices
from sixtracklib_gb300.autodiff import apply_values
from sixtracklib_gb300.particles import COL

ROWS = [COL[c] for c in ("x", "px", "y", "py", "zeta", "delta")]
SIGMA = np.array([1e-3, 1e-5, 1e-3, 1e-5, 0.05, 1e-4])


def _set_delta(block):
    f = block.view(np.float64)
    d, b0 = f[COL["delta"]], f[COL["beta0"]]
    db0 = d * b0
    ptb = np.sqrt(db0 * db0 + 2.0 * db0 * b0 + 1.0) - 1.0
    opd = 1.0 + d
    f[COL["rvv"]] = opd / (1.0 + ptb)
    f[COL["rpp"]] = 1.0 / opd
    f[COL["psigma"]] = ptb / (b0 * b0)


def _coords(block):
    f = block.view(np.float64)
    return np.stack([f[r] for r in ROWS])


@pytest.fixture(scope="module")
def ring():
    return lattices.learnable_fodo_ring()


@pytest.fixture(scope="module")
def beam():
    p = lattices.gaussian_particles(48, seed=3)
    blk = p.block.copy()
    f = blk.view(np.float64)
    f[COL["x"], :6] = np.linspace(0.014, 0.019, 6)  # lost within a few turns
    return blk


def test_dual_values_match_c_oracle(oracle, ring, beam):
    e, params = ring
    ref = beam.copy()
    oracle.track_until(e.cbuffer.to_image(), ref, 12)
    vals, ders, st, at, ae = dual.track_until(e, beam.copy(), 12,
                                              params=[(params[0][0], 2)])
    ri = ref.view(np.int64)
    assert np.array_equal(st, ri[COL["state"]])
    assert np.array_equal(at, ri[COL["at_turn"]])
    assert np.array_equal(ae, ri[COL["at_element"]])
    assert (st == 0).sum() >= 4
    assert np.array_equal(vals, _coords(ref))  # same arithmetic, same order


def test_dual_coordinate_derivatives_vs_finite_differences(oracle, ring, beam):
    e, _ = ring
    img = e.cbuffer.to_image()
    T = 12
    blk = beam[:, 6:].copy()  # particles that survive
    n = blk.shape[1]
    w = np.random.default_rng(0).normal(size=(6, n)) / SIGMA[:, None]
    vals, ders, st, _, _ = dual.track_until(e, blk.copy(), T)
    assert (st == 1).all()
    for c, row in enumerate(ROWS):
        h = 1e-5 * SIGMA[c]
        bp, bm = blk.copy(), blk.copy()
        bp.view(np.float64)[row] += h
        bm.view(np.float64)[row] -= h
        if row == COL["delta"]:
            _set_delta(bp)
            _set_delta(bm)
        oracle.track_until(img, bp, T)
        oracle.track_until(img, bm, T)
        g_fd = np.sum(w * (_coords(bp) - _coords(bm)), axis=0) / (2 * h)
        g_dual = np.sum(w * ders[c], axis=0)
        err = np.max(np.abs(g_dual - g_fd)) / np.max(np.abs(g_dual))
        assert err < 1e-6, (c, err)


def test_dual_strength_derivatives_vs_finite_differences(oracle, ring, beam):
    e, params = ring
    T = 12
    blk = beam[:, 6:].copy()
    n = blk.shape[1]
    w = np.random.default_rng(1).normal(size=(6, n)) / SIGMA[:, None]
    sel = [0, 7, 64, 70]  # quads (one carries a sextupole) and sextupoles
    rel_h = {0: 1e-7, 7: 1e-7, 64: 1e-3, 70: 1e-3}
    kinds = [(params[j][0], 2 * params[j][2]) for j in sel]
    vals0 = np.array([e.get(el).bal[2 * k] * factorial(k) for el, _, k in params])
    _, ders, _, _, _ = dual.track_until(e, blk.copy(), T, params=kinds)
    for jj, j in enumerate(sel):
        k = params[j][2]
        g_dual = np.sum(w * ders[6 + jj]) / factorial(k)
        h = rel_h[j] * abs(vals0[j])
        coords = []
        for s in (1.0, -1.0):
            v = vals0.copy()
            v[j] += s * h
            b = blk.copy()
            oracle.track_until(apply_values(e, params, v).cbuffer.to_image(), b, T)
            coords.append(_coords(b))
        g_fd = np.sum(w * (coords[0] - coords[1])) / (2 * h)
        assert abs(g_dual - g_fd) <= 1e-6 * abs(g_fd), (j, g_dual, g_fd)


def test_apply_values_round_trip(ring):
    e, params = ring
    vals = np.arange(1, len(params) + 1, dtype=np.float64) * 1e-3
    e2 = apply_values(e, params, vals)
    for (el, name, k), v in zip(params, vals):
        assert e2.get(el).bal[2 * k] * factorial(k) == pytest.approx(v, rel=1e-15)
    assert len(e2) == len(e)


@pytest.mark.parametrize("p0c", [7e12, 20e9])
def test_dual_field_kicks_vs_finite_differences(oracle, p0c):
    """4D beam-beam, coasting / q-Gaussian / interpolated space charge and the
    RF multipole (tests/adjoint_cases.field_ring): dual-number values equal
    the C oracle's (cerrf is the oracle's own), derivatives agree with
    central differences (h = 1e-5 of each spread) to 2e-6 of the row's
    largest entry -- the differences carry the nonlinear kicks' rounding.
    At 20 GeV the kicks' dependence on delta through rvv is resolvable in
    double precision; at 7 TeV rvv - 1 ~ delta / gamma^2 is below an ulp."""
    from .adjoint_cases import field_ring

    e, _, tables = field_ring()
    img = e.cbuffer.to_image()
    T = 6
    blk = lattices.gaussian_particles(40, seed=7, sz=0.08, p0c=p0c).block.copy()
    ref = blk.copy()
    assert oracle.track_until(img, ref, T) == 0
    vals, ders, st, _, _ = dual.track_until(e, blk.copy(), T)
    assert np.array_equal(st, ref.view(np.int64)[COL["state"]])
    scale = np.abs(_coords(ref)).max(axis=1, keepdims=True)
    assert np.max(np.abs(vals - _coords(ref)) / scale) < 1e-14
    w = np.random.default_rng(1).normal(size=(6, blk.shape[1])) / SIGMA[:, None]
    for c, row in enumerate(ROWS):
        h = 1e-5 * SIGMA[c]
        bp, bm = blk.copy(), blk.copy()
        bp.view(np.float64)[row] += h
        bm.view(np.float64)[row] -= h
        if row == COL["delta"]:
            _set_delta(bp)
            _set_delta(bm)
        oracle.track_until(img, bp, T)
        oracle.track_until(img, bm, T)
        g_fd = np.sum(w * (_coords(bp) - _coords(bm)), axis=0) / (2 * h)
        g_dual = np.sum(w * ders[c], axis=0)
        err = np.max(np.abs(g_dual - g_fd)) / np.max(np.abs(g_dual))
        assert err < 2e-6, (c, err)
    del tables


@pytest.mark.parametrize("p0c", [7e12, 20e9])
def test_dual_beam_beam_6d_vs_finite_differences(oracle, p0c):
    """6D beam-beam (tests/adjoint_cases.bb6d_ring: round uncoupled, coupled
    elliptic and head-on elliptic strong beams, five slices each): values
    within 1e-14 of the C oracle's, derivatives within 2e-6 of central
    differences (h = 1e-5 of each spread), and the beam-beam elements move
    the gradients by far more than that."""
    from .adjoint_cases import bb6d_ring

    e, _ = bb6d_ring(p0c)
    img = e.cbuffer.to_image()
    T = 6
    blk = lattices.gaussian_particles(40, seed=7, sz=0.08, p0c=p0c).block.copy()
    ref = blk.copy()
    assert oracle.track_until(img, ref, T) == 0
    vals, ders, st, _, _ = dual.track_until(e, blk.copy(), T)
    assert np.array_equal(st, ref.view(np.int64)[COL["state"]])
    scale = np.abs(_coords(ref)).max(axis=1, keepdims=True)
    assert np.max(np.abs(vals - _coords(ref)) / scale) < 1e-14
    _, ders0, _, _, _ = dual.track_until(lattices.fodo_ring(), blk.copy(), T)
    w = np.random.default_rng(1).normal(size=(6, blk.shape[1])) / SIGMA[:, None]
    for c, row in enumerate(ROWS):
        h = 1e-5 * SIGMA[c]
        bp, bm = blk.copy(), blk.copy()
        bp.view(np.float64)[row] += h
        bm.view(np.float64)[row] -= h
        if row == COL["delta"]:
            _set_delta(bp)
            _set_delta(bm)
        oracle.track_until(img, bp, T)
        oracle.track_until(img, bm, T)
        g_fd = np.sum(w * (_coords(bp) - _coords(bm)), axis=0) / (2 * h)
        g_dual = np.sum(w * ders[c], axis=0)
        err = np.max(np.abs(g_dual - g_fd)) / np.max(np.abs(g_dual))
        assert err < 2e-6, (c, err)
        effect = np.max(np.abs(g_dual - np.sum(w * ders0[c], axis=0))) / np.max(np.abs(g_dual))
        assert effect > 1e-3, (c, effect)


def test_parameter_table():
    """The per-element table the adjoint kernel reads, and the errors for
    parameters the lattice does not have."""
    from sixtracklib_gb300.autodiff import parameter_table

    e, params = lattices.learnable_fodo_ring()
    extra = [(params[3][0], "ksl", 1), (256, "voltage"), (params[0][0], "knl", 0)]
    t = parameter_table(e, params + extra)
    n = len(params) + len(extra)
    assert t["begin"][-1] == n and t["begin"].size == len(e) + 1
    assert np.all(np.diff(t["begin"]) >= 0)
    for el in range(len(e)):
        ids = t["entry_id"][t["begin"][el]:t["begin"][el + 1]]
        assert all(t["element"][i] == el for i in ids)
        assert list(t["entry_kind"][t["begin"][el]:t["begin"][el + 1]]) == [t["kind"][i] for i in ids]
    assert t["kind"][len(params)] == 3 and t["kind"][len(params) + 1] == -1
    assert t["value"][len(params) + 1] == 6e6
    assert t["scale"][params.index(params[-1])] == 0.5  # knl[2]: bal = knl / 2!
    for bad, exc in (((0, "knl", 1), TypeError), ((1, "knl", 5), ValueError),
                     ((1, "kn", 1), ValueError), ((999, "voltage"), IndexError),
                     ((1, "voltage"), TypeError)):
        with pytest.raises(exc):
            parameter_table(e, [bad])

