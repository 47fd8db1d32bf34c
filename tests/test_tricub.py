"""The TriCub map and the map feature flags on the CPU: the oracle against
the reference's known-answer kicks and against the reference's own builds
with other feature flags (fixtures in tests/golden/, made by
tests/golden/make_golden.py --tricub; live where the reference tree is
mounted), the coefficient matrix, and the element classes' buffer layout.
"""

import contextlib
import os

import numpy as np
import pytest

from sixtracklib_gb300.beam_elements import Elements, TriCub, TriCubData
from sixtracklib_gb300.cbuffer import CBuffer

from . import tricub_cases as tc

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def load(name):
    return np.load(os.path.join(GOLDEN, name))


@contextlib.contextmanager
def flags(oracle, f):
    oracle.set_track_flags(*f)
    try:
        yield
    finally:
        oracle.set_track_flags()


def test_coefficient_matrix_is_the_inverse_hermite_constraint_matrix(oracle):
    """The oracle's coefficients (Kronecker product of the 1-D cubic Hermite
    inverse) solve the 64 tricubic constraints: value and first derivatives
    (and their mixed products) at the eight corners."""
    rng = np.random.default_rng(0)
    b = rng.normal(size=64)
    c = oracle.tricub_coefs(b)
    kinds = [(0, 0, 0), (1, 0, 0), (0, 1, 0), (0, 0, 1), (1, 1, 0), (1, 0, 1), (0, 1, 1),
             (1, 1, 1)]

    def d(n, a, t):
        return t ** n if a == 0 else (n * t ** (n - 1) if n else 0.0)

    for l, (ax, ay, az) in enumerate(kinds):
        for corner in range(8):
            cx, cy, cz = corner & 1, (corner >> 1) & 1, corner >> 2
            v = sum(c[i + 4 * j + 16 * k] * d(i, ax, cx) * d(j, ay, cy) * d(k, az, cz)
                    for i in range(4) for j in range(4) for k in range(4))
            assert abs(v - b[8 * l + corner]) < 1e-12


def test_coefficients_bit_identical_to_reference(oracle):
    from oracle.pyoracle import Oracle

    ref = Oracle.reference()
    if ref is None:
        pytest.skip("reference sources not available here")
    rng = np.random.default_rng(1)
    for scale in (1.0, 1e-9, 1e7):
        b = rng.normal(size=64) * scale
        assert np.array_equal(oracle.tricub_coefs(b), ref.tricub_coefs(b))


def test_reference_known_answer_kicks(oracle):
    """tests/python/beam_elements/test_tricub.py:9-113 with the stored kicks:
    px, py, ptau after one TriCub of length 1 within the reference's
    tolerance (np.allclose, rtol 1e-12, atol 1e-13)."""
    d = load("tricub_kicks.npz")
    e, p = tc.kicks_case(int(d["seed"]))
    b = p.block.copy()
    with flags(oracle, (2, 2, 2, 2)):
        assert oracle.track_until(e.cbuffer.to_image(), b, 1) == 0
    f = b.view(np.float64)
    got = np.stack([f[8], f[9], f[11] * f[2]], axis=1)  # ptau = psigma beta0
    np.testing.assert_allclose(got, d["kicks"], rtol=1e-12, atol=1e-13)


def test_tricub_ring_matches_reference_build(oracle):
    """FODO ring + two TriCub kicks (mirrored; shifted with dipolar
    corrections) tracked 1 and 20 turns: bit-identical to the reference's
    TriCub-enabled build."""
    d = load("ref_tricub.npz")
    for turns in (1, 20):
        b = d["initial"].copy()
        with flags(oracle, tc.FLAG_BUILDS["a"]):
            st = oracle.track_until(d["lattice"], b, turns)
        assert st == int(d[f"status_{turns}"]) == 0
        assert np.array_equal(b, d[f"final_{turns}"])


def test_tricub_fixture_lattice_is_the_case_builder():
    d = load("ref_tricub.npz")
    assert np.array_equal(tc.tricub_ring().cbuffer.to_image(), d["lattice"])
    assert np.array_equal(tc.tricub_particles(512, 21).block, d["initial"])


@pytest.mark.parametrize("build", list(tc.FLAG_BUILDS))
def test_feature_flags_match_reference_builds(oracle, build):
    """Each element alone (track_line) and the whole lattice for 3 turns
    under the reference's default build and two builds with other flags:
    skipped maps succeed, disabled ones fail, and with space charge not
    enabled the interpolated profile loses the particle (it has no case
    label then)."""
    d = load("ref_flags.npz")
    img = d["lattice"]
    with flags(oracle, tc.FLAG_BUILDS[build]):
        b = d["initial"].copy()
        assert oracle.track_until(img, b, 3) == int(d[f"until_status_{build}"])
        assert np.array_equal(b, d[f"until_{build}"])
        for k in range(d[f"line_{build}"].shape[0]):
            b = d["initial"].copy()
            assert oracle.track_line(img, b, k, k + 1) == int(d[f"line_status_{build}"][k])
            assert np.array_equal(b, d[f"line_{build}"][k]), k


def test_live_flags_and_tricub_against_reference(oracle):
    """Live against the reference's flag builds: the flag lattice with
    other particles, and the TriCub ring with other particles."""
    from oracle.pyoracle import Oracle

    if Oracle.reference() is None:
        pytest.skip("reference sources not available here")
    lat = tc.flags_lattice(seed=11)
    img = lat.cbuffer.to_image()
    p = tc.tricub_particles(128, 40)
    for build, f in tc.FLAG_BUILDS.items():
        ref = Oracle.reference(flags=None if build == "default" else build)
        a, b = p.block.copy(), p.block.copy()
        with flags(oracle, f):
            sa = oracle.track_until(img, a, 2)
        assert sa == ref.track_until(img, b, 2)
        assert np.array_equal(a, b)
    ring = tc.tricub_ring(seed=9)
    img = ring.cbuffer.to_image()
    p = tc.tricub_particles(256, 41)
    a, b = p.block.copy(), p.block.copy()
    with flags(oracle, tc.FLAG_BUILDS["a"]):
        assert oracle.track_until(img, a, 5) == 0  # every particle stays inside the grids
    assert Oracle.reference(flags="a").track_until(img, b, 5) == 0
    assert np.array_equal(a, b)


def test_outside_the_grid_fails_and_loses(oracle):
    """A particle outside the grid (the reference would read outside its
    table) fails the map and is lost where it stands; the others are
    tracked."""
    e, p = tc.kicks_case(5, n_part=8)
    p.x[3] = -1.0  # left of the grid
    p.y[5] = 1.0   # above it
    b = p.block.copy()
    with flags(oracle, (2, 2, 2, 2)):
        assert oracle.track_until(e.cbuffer.to_image(), b, 1) == -1
    assert list(b[20]) == [1, 1, 1, 0, 1, 0, 1, 1]
    assert b[18][3] == 0 and b[19][3] == 0  # at the TriCub, turn 0
    f0, f = p.block.view(np.float64), b.view(np.float64)
    assert f[8][3] == f0[8][3] and f[9][5] == f0[9][5]  # coordinates left as they were
    assert np.all(f[8][[0, 1, 2, 4, 6, 7]] != 0.0)


def test_tricub_data_table_is_a_view_of_the_buffer():
    """TriCubData's table is zero-filled at the grid's size and edits of
    ``table_addr[i]`` reach the buffer (the reference's test fills it so,
    test_tricub.py:84-94); a TriCub linked to data in the same buffer gets
    its address in every image, and reading the image back keeps the link."""
    cb = CBuffer()
    tc_elem = TriCub(cbuffer=cb, data=1, length=2.0)
    data = TriCubData(cbuffer=cb, nx=3, ny=4, nz=5, dx=0.1)
    assert data.table_addr.size == 3 * 4 * 5 * 8 and not data.table_addr.any()
    img0 = cb.to_image().copy()
    data.table_addr[7] = 2.5
    img = cb.to_image()
    assert not np.array_equal(img0, img)
    back = CBuffer.from_image(img)
    got = back.get_object(1, TriCubData)
    assert got.table_addr[7] == 2.5 and got.nx == 3 and got.dx == 0.1
    t = back.get_object(0, TriCub)
    assert t.data == 1 and t.length == 2.0
    # data_addr is the TriCubData's absolute address in the image
    base = int(img[0])
    objs = (int(img[4]) - base) // 8
    assert int(img[(int(img[objs + 2]) - base) // 8 + 7]) == int(img[objs + 2 + 3])
    assert tc_elem.data == 1
    with pytest.raises(ValueError):
        TriCubData(nx=2, ny=2, nz=2, table_addr=np.zeros(5))


def test_engine_config_keys_for_flags():
    assert tc.flags_config((2, 1, 0, 2)) == (
        "track_beambeam4d=enabled track_beambeam6d=skip track_spacecharge=disabled "
        "track_tricub=enabled")
    e = Elements()
    e.TriCub()
    assert len(e) == 1
