"""The fast arithmetic policy restated on the CPU (oracle.c built with
ORC_FAST_POLICY): how far it departs from the reference, measured without a
GPU.  The plain-ring maps take the engine's fast forms -- explicit FMAs, the
multipole's first Horner step without the zero skew products, the Goertzel
recurrence for real-coefficient multipoles of order >= 3 (or, in the second
build, the Horner kick throughout); `tests/test_gpu_parity.py` compares the
GPU's fast mode with this restatement."""

import numpy as np
import pytest

from oracle.pyoracle import Oracle
from sixtracklib_gb300 import lattices
from sixtracklib_gb300.beam_elements import Elements

from .test_gpu_parity import max_col_dev


@pytest.fixture(scope="module")
def oracles():
    return Oracle(), Oracle.fast_policy(goertzel=True), Oracle.fast_policy(goertzel=False)


def _kick_devs(ref, fast, n_lat=400, n_part=512, seed=3):
    """Relative deviation of the px / py kicks of single real-coefficient
    multipoles (orders 3-10, the benchmark ring's coefficient scales) from
    the reference's Horner kick."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n_lat):
        order = int(rng.integers(3, 11))
        knl = np.zeros(order + 1)
        knl[1] = rng.choice([-1, 1]) * rng.uniform(0.01, 0.05)
        for n in range(2, order + 1):
            knl[n] = rng.normal(0.0, 1e-4 * 10.0 ** (-n))
        e = Elements()
        e.Multipole(knl=list(knl))
        img = e.cbuffer.to_image()
        p = lattices.gaussian_particles(n_part, seed=int(rng.integers(1 << 30)), sx=5e-3, sy=5e-3)
        # chi = 0.5: a kick well above the rounding of px + kick
        p.block[15] = np.full(n_part, 0.5).view(np.uint64)
        a, b = p.block.copy(), p.block.copy()
        ref.track_line(img, a, 0, 1, False)
        fast.track_line(img, b, 0, 1, False)
        k0 = p.block[8:10].view(np.float64)
        ka = a[8:10].view(np.float64) - k0
        kb = b[8:10].view(np.float64) - k0
        # relative to the kick, with a floor of 1e-3 of the sample's largest
        # (a kick that nearly vanishes, y ~ 0 for py, has no relative scale)
        floor = 1e-3 * np.max(np.abs(ka), axis=1, keepdims=True)
        out.append(np.abs(kb - ka) / np.maximum(np.abs(ka), floor))
    return np.concatenate(out, axis=1)


def test_goertzel_kick_rounds_like_the_horner_kick(oracles):
    """Per-component deviation of the kick from the reference's Horner: the
    Goertzel form's distribution matches the FMA Horner's (rms within 1.5x,
    99.99 % of the kicks within 5e-15); its worst kicks, where the real
    part's terms nearly cancel, reach ~2e-14 of the kick (the Horner form's
    ~1e-14) -- some 1e-21 of a momentum of the benchmark's scale."""
    ref, goertzel, horner = oracles
    dg, dh = _kick_devs(ref, goertzel), _kick_devs(ref, horner)
    rg, rh = float(np.sqrt(np.mean(dg ** 2))), float(np.sqrt(np.mean(dh ** 2)))
    qg, qh = float(np.quantile(dg, 0.9999)), float(np.quantile(dh, 0.9999))
    print(f"kick deviation rms: Goertzel {rg:.3e}, FMA Horner {rh:.3e}; "
          f"99.99 % {qg:.2e} / {qh:.2e}; max {dg.max():.2e} / {dh.max():.2e}")
    assert rg < 1.5 * rh
    assert qg < 5e-15 and qh < 5e-15
    assert dg.max() < 5e-14 and dh.max() < 5e-14


@pytest.mark.parametrize("goertzel", [True, False])
def test_fast_policy_on_the_20k_ring(oracles, goertzel):
    """2,048 polar-grid protons on the 20k ring: identical losses and
    counters; x, y, px, py and the energy columns within 1e-13 of their
    column scale after 1 and 5 turns; zeta -- whose column starts at zero --
    within 1e-12 after one turn and 2e-12 after five."""
    ref, fast = oracles[0], oracles[1 if goertzel else 2]
    lat = lattices.synthetic_ring().cbuffer.to_image()
    p = lattices.polar_grid_particles(2048, seed=5)
    for turns, zeta_tol in ((1, 1e-12), (5, 2e-12)):
        exp, got = p.block.copy(), p.block.copy()
        assert ref.track_until(lat, exp, turns) == 0
        assert fast.track_until(lat, got, turns) == 0
        assert np.array_equal(got[17:], exp[17:])
        no_zeta = got.copy()
        no_zeta[10] = exp[10]
        dev, dz = max_col_dev(no_zeta, exp), max_col_dev(got, exp)
        print(f"{'Goertzel' if goertzel else 'Horner'} {turns} turns: zeta {dz:.2e}, "
              f"other columns {dev:.2e}")
        assert dev <= 1e-13
        assert dz <= zeta_tol


@pytest.mark.parametrize("amp", [1e-3, 0.1, 0.99])
@pytest.mark.parametrize("order", [3, 10, 40])
def test_goertzel_kick_at_large_amplitudes_and_orders(oracles, amp, order):
    """The Goertzel form keeps its accuracy where the high orders matter:
    coefficients b_n ~ 10^-n (not 10^-n / n!), coordinates up to the global
    aperture (1 m), orders up to 40; every kick within 1e-15 of the
    sample's largest, as the FMA Horner form's."""
    ref, goertzel, horner = oracles
    rng = np.random.default_rng(order * 100 + int(amp * 1000))
    for trial in range(5):
        knl = np.zeros(order + 1)
        knl[1] = 0.03
        for n in range(2, order + 1):
            knl[n] = rng.normal(0.0, 1.0) * 10.0 ** (-n)
        e = Elements()
        e.Multipole(knl=list(knl))
        img = e.cbuffer.to_image()
        blk = lattices.gaussian_particles(256, seed=trial, sx=amp, sy=amp).block
        blk[15] = np.full(256, 0.5).view(np.uint64)  # chi
        a, b, c = blk.copy(), blk.copy(), blk.copy()
        ref.track_line(img, a, 0, 1, False)
        goertzel.track_line(img, b, 0, 1, False)
        horner.track_line(img, c, 0, 1, False)
        k0 = blk[8:10].view(np.float64)
        ka = a[8:10].view(np.float64) - k0
        scale = np.max(np.abs(ka), axis=1, keepdims=True)
        for other in (b, c):
            kick = other[8:10].view(np.float64) - k0
            assert np.max(np.abs(kick - ka) / scale) < 1e-15
