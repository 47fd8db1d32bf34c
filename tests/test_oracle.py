"""The oracle pinned against the reference.

* against the reference's own known-answer data (converted into
  tests/golden/ by tests/golden/make_golden.py): the pysixtrack
  element-by-element dump of `bbsimple`, the 1000-drift and 1000-exact-drift
  tracking data, the Faddeeva table;
* against outputs of the reference's own tracking code (oracle/_ref) stored
  as fixtures -- bit-identical;
* live against oracle/_ref where the reference tree is mounted: every
  element kind, every loop mode, bit-identical.
"""

import os

import numpy as np
import pytest

from oracle.pyoracle import EbeConfig
from sixtracklib_gb300 import lattices
from sixtracklib_gb300.beam_elements import Elements

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
REAL_COLS = [5, 6, 7, 8, 9, 10, 11, 12, 13, 14]  # s x y px py zeta psigma delta rpp rvv


def load(name):
    return np.load(os.path.join(GOLDEN, name))


def test_bbsimple_element_by_element_dump(oracle):
    """pysixtrack dump of the bbsimple lattice (Drift, Multipole, Cavity, BB4D,
    BB6D): state i tracked through element i reproduces state i+1
    (reference test: common/test_track_c99.cpp:389-630, tolerance there 1e-13)."""
    d = load("bbsimple.npz")
    lat, states = d["lattice"], d["states"]
    n_elem = states.shape[0] - 1
    worst = 0.0
    for i in range(n_elem):
        b = states[i].copy()
        b[20] = 1  # the dump marks state only on the final record
        st = oracle.track_line(lat, b, i, i + 1, False)
        assert st == 0
        got = b[[6, 7, 8, 9, 10, 12]].view(np.float64)
        exp = states[i + 1][[6, 7, 8, 9, 10, 12]].view(np.float64)
        worst = max(worst, float(np.max(np.abs(got - exp))))
    assert worst <= 1e-15, worst


@pytest.mark.parametrize("name,tol", [("drift", np.finfo(float).eps), ("driftexact", 5e-14)])
def test_drift_known_answer(oracle, name, tol):
    """test_track_be_drift(exact)_data.bin: 1000 drifts, one turn
    (common/test_track_c99.cpp:298-358)."""
    d = load(f"{name}.npz")
    b = d["initial"].copy()
    assert oracle.track_until(d["lattice"], b, 1) == 0
    got = b[REAL_COLS].view(np.float64)
    exp = d["expected"][REAL_COLS].view(np.float64)
    assert np.max(np.abs(got - exp)) <= tol


def test_faddeeva_table(oracle):
    """test_faddeeva_errorfn_data.bin: w(z) on [-5.33,5.33] x [-4.29,4.29].
    The CERN algorithm is an approximation: the table (an exact w) agrees to
    ~5e-10 relative."""
    pts = load("faddeeva.npz")["points"]
    worst = 0.0
    for re, im, wr, wi in pts:
        a, b = oracle.cerrf(re, im)
        err = abs(complex(a, b) - complex(wr, wi)) / max(abs(complex(wr, wi)), 1e-300)
        worst = max(worst, err)
    assert worst < 1e-9, worst


def _lattice_for(name):
    if name == "synthetic":
        return lattices.synthetic_ring().cbuffer.to_image()
    return None


@pytest.mark.parametrize("case", ["fodo", "synthetic", "bbsc", "bbsc_elliptic", "misc"])
def test_oracle_matches_reference_fixtures(oracle, case):
    d = load(f"ref_{case}.npz")
    lat = d["lattice"] if "lattice" in d else _lattice_for(case)
    import hashlib

    assert hashlib.sha256(np.ascontiguousarray(lat).tobytes()).hexdigest() == str(
        d["lattice_sha256"]), "lattice generator changed: regenerate tests/golden"
    mons = [np.zeros_like(d["monitor0"])] if "monitor0" in d else None
    b = d["initial"].copy()
    st = oracle.track_until(lat, b, int(d["turns"]), monitors=mons)
    assert st == int(d["status"])
    assert np.array_equal(b, d["final"])
    if mons:
        assert np.array_equal(mons[0], d["monitor0"])
    b = d["initial"].copy()
    lm = [np.zeros_like(d["monitor0"])] if "monitor0" in d else None
    n = len(lattices.synthetic_ring()) if case == "synthetic" else None
    end = 9 if n is None or n >= 9 else n
    assert oracle.track_line(lat, b, 3, end, False, monitors=lm) == int(d["line_status"])
    assert np.array_equal(b, d["line_final"])
    if "ebe_out" in d:
        cfg = EbeConfig(*[int(v) for v in d["ebe_cfg"]])
        out = np.zeros_like(d["ebe_out"])
        b = d["initial"].copy()
        em = [np.zeros_like(d["monitor0"])] if "monitor0" in d else None
        assert oracle.track_elem_by_elem(lat, b, cfg, out, 2, monitors=em) == int(d["ebe_status"])
        assert np.array_equal(b, d["ebe_final"])
        assert np.array_equal(out, d["ebe_out"])


@pytest.mark.parametrize("name", ["lhc_no_bb", "beambeam"])
def test_oracle_matches_reference_on_shipped_lattices(oracle, name):
    """The reference's shipped LHC lattices (tests/testdata/{lhc_no_bb,
    beambeam}/beam_elements.bin) tracked by the reference build: the oracle
    reproduces it bit for bit after 1 turn (all 1,024 particles) and after
    1,000 turns (a 16-particle subset, to keep the CPU suite short)."""
    import hashlib

    d = load(f"ref_shipped_{name}.npz")
    lat = d["lattice"]
    assert hashlib.sha256(np.ascontiguousarray(lat).tobytes()).hexdigest() == str(
        d["lattice_sha256"])
    b = d["initial"].copy()
    assert oracle.track_until(lat, b, 1) == int(d["status_1"])
    assert np.array_equal(b, d["final_1"])
    sub = np.ascontiguousarray(d["initial"][:, :16])
    assert oracle.track_until(lat, sub, 1000) == int(d["status_1000"])
    assert np.array_equal(sub, d["final_1000"][:, :16])


# ------------------------------------------------------------ live reference
def _random_lattice(seed):
    rng = np.random.default_rng(seed)
    e = Elements()
    for _ in range(60):
        k = rng.integers(0, 12)
        if k == 0:
            e.Drift(length=float(rng.uniform(0, 3)))
        elif k == 1:
            e.DriftExact(length=float(rng.uniform(0, 3)))
        elif k == 2:
            o = int(rng.integers(0, 6))
            e.Multipole(knl=list(rng.normal(0, 1e-3, o + 1)), ksl=list(rng.normal(0, 1e-4, o + 1)),
                        hxl=float(rng.choice([0.0, 1e-5])), hyl=float(rng.choice([0.0, -1e-5])),
                        length=float(rng.choice([0.0, 1.0])))
        elif k == 3:
            e.Cavity(voltage=float(rng.uniform(0, 1e6)), frequency=4e8, lag=float(rng.uniform(0, 360)))
        elif k == 4:
            e.XYShift(dx=float(rng.normal(0, 1e-4)), dy=float(rng.normal(0, 1e-4)))
        elif k == 5:
            e.SRotation(angle=float(rng.normal(0, 5)))
        elif k == 6:
            e.LimitRect(min_x=-0.03, max_x=0.03, min_y=-0.02, max_y=0.025)
        elif k == 7:
            e.LimitEllipse(a=0.03, b=0.02)
        elif k == 8:
            e.LimitRectEllipse(max_x=0.03, max_y=0.02, a=0.035, b=0.025)
        elif k == 9:
            e.DipoleEdge(r21=float(rng.normal(0, 1e-3)), r43=float(rng.normal(0, 1e-3)))
        elif k == 10:
            e.RFMultipole(voltage=float(rng.uniform(0, 1e4)), frequency=4e8, lag=10.0,
                          knl=[1e-7, 1e-4], ksl=[0, 1e-5], pn=[5, 10], ps=[1, 2])
        else:
            e.SCQGaussProfile(number_of_particles=1e11, bunchlength_rms=0.1, sigma_x=1e-3,
                              sigma_y=float(rng.choice([1e-3, 1.3e-3])), length=0.1,
                              q_param=float(rng.choice([1.0, 1.2, 0.8])))
    return e


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_oracle_matches_reference_live(oracle, ref_oracle, seed):
    lat = _random_lattice(seed).cbuffer.to_image()
    p = lattices.gaussian_particles(200, seed=seed, sx=5e-3, sy=5e-3, spx=1e-4, spy=1e-4)
    a, b = p.block.copy(), p.block.copy()
    assert oracle.track_until(lat, a, 8) == ref_oracle.track_until(lat, b, 8)
    assert np.array_equal(a, b)
    a, b = p.block.copy(), p.block.copy()
    assert oracle.track_line(lat, a, 5, 40, True) == ref_oracle.track_line(lat, b, 5, 40, True)
    assert np.array_equal(a, b)


def test_oracle_matches_reference_edge_cases(oracle, ref_oracle):
    """Aperture edges, pre-lost particles, mixed start turns, unknown and
    disabled element types, empty lattice."""
    e = Elements()
    e.Drift(length=1.0)
    e.LimitRect(min_x=-0.01, max_x=0.01, min_y=-0.01, max_y=0.01)
    e.Drift(length=0.0)
    lat = e.cbuffer.to_image()
    p = lattices.gaussian_particles(64, seed=4)
    x = p.x
    x[:8] = [0.01, -0.01, 0.0100000000001, 1.0, -1.0, 0.99999999, np.nan, np.inf]
    p.px[:8] = 0.0
    p.state[8:12] = 0
    p.at_turn[12:20] = [1, 2, 3, 5, 7, 9, 0, 4]
    for until in (0, 1, 5):
        a, b = p.block.copy(), p.block.copy()
        assert oracle.track_until(lat, a, until) == ref_oracle.track_until(lat, b, until)
        assert np.array_equal(a.view(np.uint64), b.view(np.uint64))
    # unknown type id and TriCub (disabled) in the middle
    for tid in (777, 261, 260, 258):
        e2 = Elements()
        e2.Drift(length=1.0)
        e2.cbuffer.add_object(tid, np.zeros(3, np.uint64))
        e2.Drift(length=1.0)
        lat2 = e2.cbuffer.to_image()
        for fn, args in ((oracle.track_until, (3,)), (oracle.track_line, (0, 3, True))):
            a, b = p.block.copy(), p.block.copy()
            rfn = getattr(ref_oracle, fn.__name__)
            assert fn(lat2, a, *args) == rfn(lat2, b, *args)
            assert np.array_equal(a, b)
    # empty lattice
    from sixtracklib_gb300 import CBuffer

    empty = CBuffer().to_image()
    a, b = p.block.copy(), p.block.copy()
    assert oracle.track_until(empty, a, 3) == ref_oracle.track_until(empty, b, 3) == -1
    assert np.array_equal(a, b)


def test_cerrf_matches_reference(oracle, ref_oracle):
    rng = np.random.default_rng(0)
    for re, im in rng.uniform(-8, 8, size=(3000, 2)):
        assert oracle.cerrf(re, im) == ref_oracle.cerrf(re, im)
    for args in [(1e-6, 2e-6, 3e-6, 3e-6, 1e-10, 0), (1e-6, -2e-6, 3e-6, 4e-6, 1e-10, 0),
                 (0.0, 0.0, 3e-6, 3e-6, 1e-10, 1), (1e-7, 2e-7, 3e-6, 2e-6, 1e-10, 0)]:
        assert oracle.fields_gauss(*args) == ref_oracle.fields_gauss(*args)


def test_oracle_matches_reference_interpolated_space_charge(oracle, ref_oracle):
    """SCInterpolatedProfile with linear, cubic and disabled line-density
    tables (host addresses, as the reference's CPU tracking reads them) and
    the fallback density; zeta spread beyond the tables' range."""
    e, tables = lattices.sc_interpolated_ring()
    lat = e.cbuffer.to_image()
    p = lattices.gaussian_particles(300, seed=2, sz=0.12)
    for turns in (1, 6):
        a, b = p.block.copy(), p.block.copy()
        assert oracle.track_until(lat, a, turns) == ref_oracle.track_until(lat, b, turns) == 0
        assert np.array_equal(a, b)
    dpx = a.view(np.float64)[8] - p.block.view(np.float64)[8]
    assert np.abs(dpx).max() > 0
    del tables

