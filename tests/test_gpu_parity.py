"""GPU parity: the CUDA tracking kernel against the oracle and the
reference's fixtures, through the C ABI.

Tolerances (the engine's contract):
* integer columns (particle_id, at_element, at_turn, state) identical;
* exact mode: bit-identical wherever no libm function is involved (drifts,
  multipoles, shifts, rotations, apertures: + - * / sqrt are correctly rounded
  on both sides); where sin/exp/pow enter (cavities, beam-beam, space charge)
  within 1e-13 of the column scale per turn-block and 1e-10 after 1000 turns;
* fast mode (explicit FMA): the same 1e-13 (1 turn) / 1e-10 (1000 turns).
"Column scale" = max |value| of the oracle's column, so coordinates that
cross zero are judged against their amplitude.
"""

import ctypes as C
import os

import numpy as np
import pytest

from oracle.pyoracle import EbeConfig
from sixtracklib_gb300 import lattices
from sixtracklib_gb300.beam_elements import Elements

from .deviation import amplitude_dev

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("GPU tests need a CUDA device")
    return torch


def run_device(torch, lattice, block, until=None, line=None, mode="exact"):
    from sixtracklib_gb300.device import DeviceTracker

    trk = DeviceTracker(lattice, config=f"mode={mode}")
    cols = torch.from_numpy(block.copy().view(np.int64)).cuda()
    if line is not None:
        st = trk.track_line(cols, *line)
    else:
        st = trk.track_until(cols, until)
    torch.cuda.synchronize()
    return st, cols.cpu().numpy().view(np.uint64)


def max_col_dev(got, exp):
    g = got[:17].view(np.float64)
    e = exp[:17].view(np.float64)
    both_nan = np.isnan(g) & np.isnan(e)
    scale = np.maximum(np.nanmax(np.abs(np.where(np.isfinite(e), e, 0)), axis=1, keepdims=True),
                       1e-300)
    d = np.where(both_nan, 0.0, np.abs(g - e) / scale)
    return float(np.nanmax(d)) if d.size else 0.0


def assert_fast_parity(got, exp, tol, zeta_tol):
    """The fast policy on polar-grid samples, whose particles start at
    zeta = 0: zeta within `zeta_tol` of its (small) column scale, every
    other column within `tol`.  The contracted drift sum and the kick's
    forms move the rounding of 1 + (xp^2 + yp^2) / 2 at scale 1 for a few
    large-amplitude particles per turn, about 2e-16 m of zeta each, 1e-12 of
    a zeta column that spans 2.5e-4 m (tests/test_fast_policy_cpu.py
    measures the same on the CPU)."""
    assert_parity(got, exp, tol=zeta_tol)
    no_zeta = got.copy()
    no_zeta[10] = exp[10]
    dev = max_col_dev(no_zeta, exp)
    assert dev <= tol, f"columns other than zeta: {dev:.3e}"


def assert_parity(got, exp, tol, bit_exact=False):
    assert np.array_equal(got[17:], exp[17:]), "particle ids / at_element / at_turn / state differ"
    if bit_exact:
        diff = np.nonzero((got != exp).any(axis=1))[0]
        assert diff.size == 0, f"columns {diff} not bit-identical"
    else:
        dev = max_col_dev(got, exp)
        assert dev <= tol, f"max deviation {dev:.3e} > {tol:.1e}"


_CACHE = {}


def load(name):
    return np.load(os.path.join(GOLDEN, name))


# ----------------------------------------------------- reference fixtures
@pytest.mark.parametrize("mode", ["exact", "fast"])
@pytest.mark.parametrize("case", ["fodo", "synthetic", "bbsc", "bbsc_elliptic", "misc"])
def test_reference_fixture_until(torch_cuda, case, mode):
    d = load(f"ref_{case}.npz")
    lat = d["lattice"] if "lattice" in d else lattices.synthetic_ring().cbuffer.to_image()
    st, got = run_device(torch_cuda, lat, d["initial"], until=int(d["turns"]), mode=mode)
    assert st == int(d["status"])
    assert_parity(got, d["final"], tol=1e-12)


@pytest.mark.parametrize("mode", ["exact", "fast"])
@pytest.mark.parametrize("case", ["fodo", "bbsc", "misc"])
def test_reference_fixture_line(torch_cuda, case, mode):
    d = load(f"ref_{case}.npz")
    # the monitor in `misc` stores nothing here: the device path gets no output
    lat = d["lattice"]
    st, got = run_device(torch_cuda, lat, d["initial"], line=(3, 9, False), mode=mode)
    assert st == int(d["line_status"])
    assert_parity(got, d["line_final"], tol=1e-13)


@pytest.mark.parametrize("case", ["fodo", "misc"])
def test_reference_fixture_elem_by_elem_free_function(torch_cuda, case):
    """st_Track_all_particles_element_by_element_until_turn with an explicit
    config and generic-address outputs (track/track.h:672-777)."""
    from tests import capi

    d = load(f"ref_{case}.npz")
    L = capi.lib()
    lat = d["lattice"]
    be = capi.c_buffer_from_image(lat)
    blk = d["initial"].copy()
    sp = capi.particles_view(blk)
    cfg = capi.StElemByElemConfig(*[int(v) for v in d["ebe_cfg"]], 0)
    out = np.zeros_like(d["ebe_out"])
    ga = capi.generic_addr(out)
    cfg.out_store_addr = C.addressof(ga)
    # the misc lattice carries a BeamMonitor with a placeholder out_address:
    # give it a real generic-address output (as the reference's test does)
    mon_keep = None
    if "ebe_monitor0" in d:
        mon = np.zeros_like(d["ebe_monitor0"])
        mga = capi.generic_addr(mon)
        mon_keep = (mon, mga)
        n = L.st_Buffer_get_num_of_objects(be)
        for i in range(n):
            o = C.cast(L.st_Buffer_get_const_object(be, i), C.POINTER(C.c_uint64))
            if o[1] == 10:
                m = C.cast(o[0], C.POINTER(C.c_uint64))
                m[3] = C.addressof(mga)
    st = L.st_Track_all_particles_element_by_element_until_turn(C.byref(sp), C.byref(cfg), be, 2)
    L.st_Buffer_delete(be)
    assert st == int(d["ebe_status"]), _err()
    assert_parity(blk, d["ebe_final"], tol=1e-13)
    assert_parity(out, d["ebe_out"], tol=1e-13)
    if mon_keep is not None:
        assert_parity(mon_keep[0], d["ebe_monitor0"], tol=1e-13)


def _err():
    from sixtracklib_gb300 import _native

    return _native.last_error()


# --------------------------------------------------------- exact-mode bits
def test_exact_mode_bit_identical_without_libm(torch_cuda, oracle):
    """20k-element ring without cavities: drifts, multipoles (order 1-10),
    shifts, rotations, elliptic apertures; exact mode reproduces the
    reference arithmetic bit for bit, losses included."""
    e = lattices.synthetic_ring(n_cav=0)
    lat = e.cbuffer.to_image()
    p = lattices.polar_grid_particles(4096, seed=21)
    exp = p.block.copy()
    assert oracle.track_until(lat, exp, 3) == 0
    st, got = run_device(torch_cuda, lat, p.block, until=3, mode="exact")
    assert st == 0
    assert_parity(got, exp, 0.0, bit_exact=True)
    lost = int((exp[20].view(np.int64) == 0).sum())
    assert 0 < lost < 4096


def test_exact_mode_bit_identical_line_and_misc(torch_cuda, oracle):
    e = Elements()
    for _ in range(20):
        e.Drift(length=1.3)
        e.DriftExact(length=0.7)
        e.Multipole(knl=[1e-5, 0.01, 0.02, 0.3], ksl=[0.0, 1e-4], hxl=1e-6, length=1.0)
        e.SRotation(angle=3.0)
        e.XYShift(dx=1e-5, dy=-2e-5)
        e.DipoleEdge(r21=1e-3, r43=-1e-3)
        e.Multipole(knl=[0.0, -0.01])
        e.LimitRectEllipse(max_x=0.02, max_y=0.015, a=0.025, b=0.02)
        e.LimitRect(min_x=-0.019, max_x=0.02, min_y=-0.02, max_y=0.014)
    lat = e.cbuffer.to_image()
    p = lattices.gaussian_particles(3000, seed=3, sx=4e-3, sy=4e-3, spx=1e-4, spy=1e-4)
    for args in ((0, len(e), True), (17, 93, False)):
        exp = p.block.copy()
        st0 = oracle.track_line(lat, exp, *args)
        st, got = run_device(torch_cuda, lat, p.block, line=args, mode="exact")
        assert st == st0
        assert_parity(got, exp, 0.0, bit_exact=True)
    exp = p.block.copy()
    oracle.track_until(lat, exp, 25)
    st, got = run_device(torch_cuda, lat, p.block, until=25, mode="exact")
    assert_parity(got, exp, 0.0, bit_exact=True)


# ------------------------------------------------------ long-run tolerance
@pytest.mark.parametrize("mode", ["exact", "fast"])
def test_fodo_ring_10k_particles_1000_turns(torch_cuda, oracle, mode):
    """The plain FODO ring at full size (10,000 protons, 1000 turns):
    regular orbits within 1e-10, identical loss flags / turn counters."""
    lat = lattices.fodo_ring().cbuffer.to_image()
    p = lattices.gaussian_particles(10_000, seed=2024)
    exp = p.block.copy()
    assert oracle.track_until(lat, exp, 1000) == 0
    st, got = run_device(torch_cuda, lat, p.block, until=1000, mode=mode)
    assert st == 0
    assert_parity(got, exp, tol=1e-10)
    med, p99, worst = amplitude_dev(got, exp, p.block)
    print(f"FODO {mode} 1000 turns: amplitude-normalised median {med:.2e}, 99% {p99:.2e}, "
          f"max {worst:.2e}")
    assert worst <= 1e-7
    # one turn: 1e-13
    exp1 = p.block.copy()
    oracle.track_until(lat, exp1, 1)
    st, got1 = run_device(torch_cuda, lat, p.block, until=1, mode=mode)
    assert_parity(got1, exp1, tol=1e-13)


@pytest.mark.parametrize("mode", ["exact", "fast"])
def test_synthetic_ring_sample(torch_cuda, oracle, mode):
    """2,048 polar-grid protons, 5 turns of the 20k ring.  Exact mode within
    1e-12 of every column's scale.  Fast mode: the particles start at
    zeta = 0, so the zeta column's scale is small (2.5e-4 m after a turn),
    and the contracted drift sum moves the rounding of 1 + (xp^2 + yp^2) / 2
    at scale 1 for a few large-amplitude particles per turn (about 2e-16 m
    of zeta each): zeta sits at 0.76e-12 of its column after one turn and
    0.9-1.0e-12 after five (a CPU restatement of the fast policy gives the
    same figures, with the Horner and with the Goertzel form of the kick),
    so it is held to 2e-12 and every other column to 1e-13
    (`tests/test_fast_policy_cpu.py` measures the same on the CPU)."""
    lat = lattices.synthetic_ring().cbuffer.to_image()
    p = lattices.polar_grid_particles(2048, seed=5)
    exp = p.block.copy()
    oracle.track_until(lat, exp, 5)
    st, got = run_device(torch_cuda, lat, p.block, until=5, mode=mode)
    assert st == 0
    if mode == "exact":
        assert_parity(got, exp, tol=1e-12)
    else:
        assert_fast_parity(got, exp, tol=1e-13, zeta_tol=2e-12)


def test_fast_mode_equals_its_cpu_restatement(torch_cuda):
    """The GPU's fast policy and its CPU restatement (oracle.c with
    ORC_FAST_POLICY=1: the same FMAs, zero-skew first Horner step and
    Goertzel kick) agree bit for bit on the 20k ring without its cavities
    (whose sin() is CUDA's on one side and the host libm's on the other):
    2,048 polar-grid protons, 5 turns, losses included, every column."""
    from oracle.pyoracle import Oracle

    lat = lattices.synthetic_ring(n_cav=0).cbuffer.to_image()
    p = lattices.polar_grid_particles(2048, seed=5)
    exp = p.block.copy()
    assert Oracle.fast_policy(goertzel=True).track_until(lat, exp, 5) == 0
    st, got = run_device(torch_cuda, lat, p.block, until=5, mode="fast")
    assert st == 0
    assert_parity(got, exp, 0.0, bit_exact=True)


@pytest.mark.parametrize("mode", ["exact", "fast"])
def test_synthetic_ring_1000_turns(torch_cuda, oracle, mode):
    """The 20,000-element ring over 1000 turns on a strided 1,024-particle
    sample of the benchmark's polar grid (amplitudes 0-20 sigma, so particles
    are lost on the way): loss flags, at_element and at_turn identical,
    coordinates within 1e-10 of the column scale; the amplitude-normalised
    deviation of each surviving particle reported beside it."""
    if "synthetic_1000" not in _CACHE:  # the oracle run serves both modes
        lat = lattices.synthetic_ring().cbuffer.to_image()
        full = lattices.polar_grid_particles(1_000_000, seed=99)
        blk = np.ascontiguousarray(full.block[:, ::977][:, :1024])
        exp = blk.copy()
        assert oracle.track_until(lat, exp, 1000) == 0
        _CACHE["synthetic_1000"] = (lat, blk, exp)
    lat, blk, exp = _CACHE["synthetic_1000"]
    st, got = run_device(torch_cuda, lat, blk, until=1000, mode=mode)
    assert st == 0
    lost = int((exp.view(np.int64)[20] == 0).sum())
    assert 0 < lost < blk.shape[1]
    assert_parity(got, exp, tol=1e-10)
    alive = exp.view(np.int64)[20] == 1
    med, p99, worst = amplitude_dev(got[:, alive], exp[:, alive], blk[:, alive])
    print(f"synthetic ring {mode} 1000 turns, {int(alive.sum())} survivors: amplitude-normalised "
          f"median {med:.2e}, 99% {p99:.2e}, max {worst:.2e}")
    assert worst <= 1e-7


@pytest.mark.parametrize("elliptic", [False, True])
def test_beam_beam_space_charge_ring(torch_cuda, oracle, elliptic):
    """FODO ring + BB6D (21 slices) + BB4D + 200 q-Gaussian space-charge
    kicks: 1e-13 after one turn, 1e-10 after 20 (the beam-beam kicks amplify
    last-bit differences of exp() between CUDA and the host libm)."""
    lat = lattices.bb_sc_ring(elliptic=elliptic).cbuffer.to_image()
    p = lattices.gaussian_particles(1024, seed=17, sx=2e-5, sy=2e-5)
    for turns, tol in ((1, 1e-13), (20, 1e-10)):
        exp = p.block.copy()
        oracle.track_until(lat, exp, turns)
        for mode in ("exact", "fast"):
            st, got = run_device(torch_cuda, lat, p.block, until=turns, mode=mode)
            assert st == 0
            assert_parity(got, exp, tol=tol)


@pytest.mark.parametrize("elliptic,turns", [(False, 100), (True, 20)])
def test_beam_beam_space_charge_full_size(torch_cuda, oracle, elliptic, turns):
    """The beam-beam and space-charge mix at its full size, 262,144 Gaussian
    protons: a strided sample of 1,024 agrees with the oracle within 1e-10
    (loss flags and counters identical), and a particle's result does not
    depend on its slot (a permuted block gives the permuted result, bit for
    bit)."""
    torch = torch_cuda
    from sixtracklib_gb300.device import DeviceTracker

    e = lattices.bb_sc_ring(elliptic=elliptic)
    trk = DeviceTracker(e, config="mode=exact")
    p = lattices.gaussian_particles(262144, seed=41)
    base = torch.from_numpy(p.block.copy().view(np.int64)).cuda()
    a = base.clone()
    assert trk.track_until(a, turns) == 0
    perm = torch.randperm(base.shape[1], device=base.device)
    c = base[:, perm].contiguous()
    assert trk.track_until(c, turns) == 0
    assert torch.equal(c, a[:, perm])
    idx = np.arange(0, 262144, 256)
    sample = p.block[:, idx].copy()
    assert oracle.track_until(e.cbuffer.to_image(), sample, turns) == 0
    assert_parity(a.cpu().numpy().view(np.uint64)[:, idx], sample, tol=1e-10)


@pytest.mark.parametrize("sigmas", [(2e-3, 1e-3), (1e-3, 2.5e-3), (1.5e-3, 1.5e-3)])
def test_gaussian_field_kicks(torch_cuda, oracle, sigmas):
    """The Gaussian field itself, one 4D beam-beam element with a strong
    beam: particles at rest in px, py on a grid out to 40 sigma (both
    branches of the Faddeeva function, the round formula for equal sizes),
    so px, py after the element are the kicks.  The device evaluates the
    CERN algorithm's truncated continued fraction and series in a
    division-free form whose values differ from the reference's
    term-by-term loop by rounding (<= 3.2e-15 relative).  Near the centre
    the field is the difference of two nearly equal Faddeeva terms, which
    amplifies any rounding difference by ~1 / r; so each kick must agree
    within 1e-13 of its magnitude, or of a tenth of the largest kick where
    it is smaller (inside ~0.2 sigma)."""
    sx, sy = sigmas
    e = Elements()
    e.BeamBeam4D(charge=1e13, sigma_x=sx, sigma_y=sy, beta_r=1.0, min_sigma_diff=1e-10,
                 x_bb=0.0, y_bb=0.0, d_px=0.0, d_py=0.0, enabled=1.0)
    lat = e.cbuffer.to_image()
    r = np.concatenate([np.linspace(0.01, 6.0, 24), np.geomspace(6.0, 40.0, 8)])
    ang = np.linspace(0.0, 2 * np.pi, 17)[:-1] + 0.1
    xs = (r[:, None] * np.cos(ang)[None, :] * sx).ravel()
    ys = (r[:, None] * np.sin(ang)[None, :] * sy).ravel()
    p = lattices.gaussian_particles(xs.size, seed=2)
    p.x[:] = xs
    p.y[:] = ys
    p.px[:] = 0.0
    p.py[:] = 0.0
    exp = p.block.copy()
    assert oracle.track_until(lat, exp, 1) == 0
    f = exp.view(np.float64)
    kick = np.hypot(f[8], f[9])
    assert kick.min() > 0
    scale = np.maximum(kick, 0.1 * kick.max())
    for mode in ("exact", "fast"):
        st, got = run_device(torch_cuda, lat, p.block, until=1, mode=mode)
        assert st == 0
        g = got.view(np.float64)
        err = np.hypot(g[8] - f[8], g[9] - f[9]) / scale
        assert err.max() < 1e-13, (mode, float(err.max()))


def test_interpolated_space_charge(torch_cuda, oracle):
    """SCInterpolatedProfile (linear / cubic / disabled tables and the
    fallback density): 1e-13 after one turn, 1e-10 after 20."""
    e, tables = lattices.sc_interpolated_ring()
    lat = e.cbuffer.to_image()
    p = lattices.gaussian_particles(1024, seed=23, sz=0.12)
    for turns, tol in ((1, 1e-13), (20, 1e-10)):
        exp = p.block.copy()
        assert oracle.track_until(lat, exp, turns) == 0
        for mode in ("exact", "fast"):
            st, got = run_device(torch_cuda, lat, p.block, until=turns, mode=mode)
            assert st == 0
            assert_parity(got, exp, tol=tol)
    del tables


def test_interpolated_space_charge_large_tables(torch_cuda, oracle):
    """Line-density tables of 10,000 points (cubic and linear) stay in global
    memory outside the element records: the lattice keeps the default
    1,024-word chunks and tracks like the oracle (1e-13 after one turn,
    1e-10 after 20)."""
    from sixtracklib_gb300.device import DeviceTracker
    from sixtracklib_gb300.sc_line_density import LineDensityBuffer

    tables = LineDensityBuffer()
    z = np.linspace(-0.4, 0.4, 10_000)
    prof = np.exp(-0.5 * (z / 0.1) ** 2) * (1 + 0.05 * np.sin(40 * z)) * 1e12
    dz = float(z[1] - z[0])
    idx = [tables.add(prof, z0=-0.4, dz=dz, method="cubic"),
           tables.add(prof * 0.9, z0=-0.4, dz=dz, method="linear")]
    e = lattices.fodo_ring()
    for k in range(6):
        e.SCInterpolatedProfile(number_of_particles=1e11, length=0.5, sigma_x=1e-3,
                                sigma_y=1e-3 if k % 2 else 1.2e-3,
                                interpol_data_addr=tables.address(idx[k % 2]),
                                line_density_prof_fallback=5e11, min_sigma_diff=1e-10)
    lat = e.cbuffer.to_image()
    assert DeviceTracker(lat).num_chunks == 1  # records stay small: one 1,024-word chunk
    p = lattices.gaussian_particles(2048, seed=29, sz=0.12)
    for turns, tol in ((1, 1e-13), (20, 1e-10)):
        exp = p.block.copy()
        assert oracle.track_until(lat, exp, turns) == 0
        for mode in ("exact", "fast"):
            st, got = run_device(torch_cuda, lat, p.block, until=turns, mode=mode)
            assert st == 0
            assert_parity(got, exp, tol=tol)
    del tables


# ------------------------------------------------------------ edge cases
def test_edge_cases(torch_cuda, oracle):
    e = Elements()
    e.Drift(length=1.0)
    e.LimitRect(min_x=-0.01, max_x=0.01, min_y=-0.01, max_y=0.01)
    e.Drift(length=0.0)
    lat = e.cbuffer.to_image()
    p = lattices.gaussian_particles(300, seed=4)
    p.x[:8] = [0.01, -0.01, 0.0100000000001, 1.0, -1.0, 0.99999999, np.nan, np.inf]
    p.px[:8] = 0.0
    p.state[8:12] = 0
    p.at_turn[12:20] = [1, 2, 3, 5, 7, 9, 0, 4]
    p.at_element[20:30] = 7
    for until in (0, 1, 5):
        exp = p.block.copy()
        s0 = oracle.track_until(lat, exp, until)
        st, got = run_device(torch_cuda, lat, p.block, until=until)
        assert st == s0
        assert_parity(got, exp, 0.0, bit_exact=True)
    for tid in (777, 261, 260):
        e2 = Elements()
        e2.Drift(length=1.0)
        e2.cbuffer.add_object(tid, np.zeros(3, np.uint64))
        e2.Drift(length=1.0)
        lat2 = e2.cbuffer.to_image()
        exp = p.block.copy()
        s0 = oracle.track_until(lat2, exp, 3)
        st, got = run_device(torch_cuda, lat2, p.block, until=3)
        assert st == s0 == -1
        assert_parity(got, exp, 0.0, bit_exact=True)
        exp = p.block.copy()
        s0 = oracle.track_line(lat2, exp, 0, 3, True)
        st, got = run_device(torch_cuda, lat2, p.block, line=(0, 3, True))
        assert st == s0
        assert_parity(got, exp, 0.0, bit_exact=True)


def test_empty_lattice_and_no_particles(torch_cuda):
    from sixtracklib_gb300 import CBuffer

    empty = CBuffer().to_image()
    p = lattices.gaussian_particles(10)
    st, got = run_device(torch_cuda, empty, p.block, until=3)
    assert st == -1
    assert np.array_equal(got, p.block)
    lat = lattices.fodo_ring().cbuffer.to_image()
    st, _ = run_device(torch_cuda, lat, np.zeros((21, 0), np.uint64), until=3)
    assert st == 0


# ------------------------------------------------ full-size properties
def test_full_size_config_properties(torch_cuda, oracle):
    """1M particles on the 20k-element ring (the benchmark workload):
    (a) 2 turns in one call == 2 calls of 1 turn, bit for bit;
    (b) the result of a particle does not depend on its slot;
    (c) a strided sample of 1024 particles agrees with the oracle (zeta,
    whose column starts at zero on the polar grid, within 2e-12 of its
    scale, every other column within 1e-13: assert_fast_parity)."""
    torch = torch_cuda
    from sixtracklib_gb300.device import DeviceTracker

    e = lattices.synthetic_ring()
    trk = DeviceTracker(e.cbuffer, config="mode=fast")
    p = lattices.polar_grid_particles(1_000_000)
    base = torch.from_numpy(p.block.copy().view(np.int64)).cuda()
    a = base.clone()
    assert trk.track_until(a, 2) == 0
    b = base.clone()
    assert trk.track_until(b, 1) == 0
    assert trk.track_until(b, 2) == 0
    assert torch.equal(a, b)
    perm = torch.randperm(base.shape[1], device=base.device)
    c = base[:, perm].contiguous()
    assert trk.track_until(c, 2) == 0
    assert torch.equal(c, a[:, perm])
    idx = np.arange(0, 1_000_000, 977)[:1024]
    sample = p.block[:, idx].copy()
    oracle.track_until(e.cbuffer.to_image(), sample, 2)
    got = a.cpu().numpy().view(np.uint64)[:, idx]
    assert_fast_parity(got, sample, tol=1e-13, zeta_tol=2e-12)


def test_trackjob_until_line_collect(torch_cuda, oracle):
    """Python TrackJob over the C ABI (python/sixtracklib/trackjob.py)."""
    from sixtracklib_gb300 import ParticlesSet
    from sixtracklib_gb300.trackjob import TrackJob

    e = lattices.fodo_ring()
    ps = ParticlesSet()
    p = ps.Particles(num_particles=500)
    q = lattices.gaussian_particles(500, seed=8)
    p.set_block(q.block)
    job = TrackJob(e, ps, config_str="mode=exact")
    job.track_until(20)
    job.collect_particles()
    exp = q.block.copy()
    oracle.track_until(e.cbuffer.to_image(), exp, 20)
    assert_parity(p.block.copy(), exp, tol=1e-13)
    job.track_line(0, 100, False)
    job.collect()
    oracle.track_line(e.cbuffer.to_image(), exp, 0, 100, False)
    assert_parity(p.block.copy(), exp, tol=1e-13)
    with pytest.raises(RuntimeError):
        TrackJob(e, ps, arch="opencl")


def test_trackjob_stored_buffers_and_address_assignment(torch_cuda, oracle):
    """Line-density tables in a stored buffer assigned to interpolated
    space-charge kicks through the TrackJob (sc_line_density.py:113-150,
    trackjob.py:1943-2035), as the reference's space-charge examples do;
    a strength edited after the job was made reaches the engine on
    push_beam_elements."""
    from sixtracklib_gb300 import ParticlesSet
    from sixtracklib_gb300.sc_line_density import LineDensityProfileData_create_buffer_assignment
    from sixtracklib_gb300.trackjob import TrackJob

    z = np.linspace(-0.3, 0.3, 41)
    prof = np.exp(-0.5 * (z / 0.1) ** 2) * 1e12
    tables = Elements()
    tables.LineDensityProfileData(values=prof, z0=-0.3, dz=float(z[1] - z[0]), method="linear",
                                  capacity=48)
    tables.LineDensityProfileData(values=prof * 1.1, z0=-0.3, dz=float(z[1] - z[0]),
                                  method="cubic")
    e = lattices.fodo_ring()
    first = len(e)
    for k in range(6):
        e.SCInterpolatedProfile(number_of_particles=1e11, length=0.5, sigma_x=1e-3,
                                sigma_y=1.2e-3 if k % 2 else 1e-3, interpol_data_addr=0,
                                line_density_prof_fallback=5e11, min_sigma_diff=1e-10)
    ps = ParticlesSet()
    p = ps.Particles(num_particles=512)
    q = lattices.gaussian_particles(512, seed=6, sz=0.12)
    p.set_block(q.block)
    job = TrackJob(e, ps, config_str="mode=exact")
    bid = job.add_stored_buffer(cbuffer=tables)
    assert bid == 1024 and job.num_stored_buffers == 1
    assert job.stored_buffer(bid).cbuffer is tables.cbuffer
    for k in range(6):
        assert LineDensityProfileData_create_buffer_assignment(job, first + k, bid, k % 2)
    assert not LineDensityProfileData_create_buffer_assignment(job, first, bid, 0)
    assert job.num_assign_items(2, bid) == 6 and job.total_num_assign_items == 6
    job.commit_address_assignments()
    job.assign_all_addresses()
    assert job.track_until(5) == 0
    job.collect_particles()
    exp = q.block.copy()
    assert oracle.track_until(e.cbuffer.to_image(), exp, 5) == 0
    assert_parity(p.block.copy(), exp, tol=1e-13)
    fallback = q.block.copy()
    e_fb = lattices.fodo_ring()
    for k in range(6):
        e_fb.SCInterpolatedProfile(number_of_particles=1e11, length=0.5, sigma_x=1e-3,
                                   sigma_y=1.2e-3 if k % 2 else 1e-3, interpol_data_addr=0,
                                   line_density_prof_fallback=5e11, min_sigma_diff=1e-10)
    oracle.track_until(e_fb.cbuffer.to_image(), fallback, 5)
    assert max_col_dev(p.block.copy(), fallback) > 1e-9  # the tables were used
    e.get(1).set_knl(0.052, 1)
    job.push_beam_elements()
    assert job.track_until(10) == 0
    job.collect_particles()
    assert oracle.track_until(e.cbuffer.to_image(), exp, 10) == 0
    assert_parity(p.block.copy(), exp, tol=1e-12)
    # reset on fresh particles: the stored tables and their assignment stay
    ps2 = ParticlesSet()
    p2 = ps2.Particles(num_particles=256)
    q2 = lattices.gaussian_particles(256, seed=7, sz=0.12)
    p2.set_block(q2.block)
    job.reset(e, ps2)
    assert job.num_stored_buffers == 1 and job.total_num_assign_items == 6
    assert job.track_until(4) == 0
    job.collect_particles()
    exp2 = q2.block.copy()
    assert oracle.track_until(e.cbuffer.to_image(), exp2, 4) == 0
    assert_parity(p2.block.copy(), exp2, tol=1e-13)


def test_trackjob_beam_monitor_and_elem_by_elem_output(torch_cuda, oracle):
    """Output buffer: elem-by-elem store first, then one Particles object per
    BeamMonitor (output/output_buffer.c:288-360)."""
    from sixtracklib_gb300 import ParticlesSet
    from sixtracklib_gb300.trackjob import TrackJob

    e = lattices.fodo_ring()
    e.BeamMonitor(num_stores=5, start=0, skip=2, is_rolling=1, is_turn_ordered=1)
    ps = ParticlesSet()
    p = ps.Particles(num_particles=64)
    q = lattices.gaussian_particles(64, seed=12)
    p.set_block(q.block)
    job = TrackJob(e, ps, until_turn_elem_by_elem=2, config_str="mode=exact")
    assert job.has_elem_by_elem_output and job.has_beam_monitor_output
    assert job.elem_by_elem_output_offset == 0 and job.beam_monitor_output_offset == 1
    job.track_elem_by_elem(2)
    job.track_until(12)
    job.collect()
    out = job.output.cbuffer
    ebe = out.get_object(0).block.copy()
    mon = out.get_object(1).block.copy()
    # oracle with the same configuration
    lat = job.beam_elements_buffer.to_image()
    ne = len(e)
    cfg = EbeConfig(0, 64, ne, 2, 0, 0, 0, 63, ne - 1, 1, 1)
    exp = q.block.copy()
    exp_ebe = np.zeros_like(ebe)
    lat_mon = e.cbuffer.objects[-1].words.copy()
    # enable the monitor's store in the oracle's copy of the lattice
    from sixtracklib_gb300 import CBuffer

    cb = CBuffer.from_image(lat)
    cb.objects[-1].words[3] = 1
    cb.objects[-1].words[4] = 63
    cb.objects[-1].words[5] = 0
    del lat_mon
    img = cb.to_image()
    exp_mon = np.zeros_like(mon)
    oracle.track_elem_by_elem(img, exp, cfg, exp_ebe, 2, monitors=[exp_mon])
    oracle.track_until(img, exp, 12, monitors=[exp_mon])
    assert_parity(p.block.copy(), exp, tol=1e-13)
    assert_parity(ebe, exp_ebe, tol=1e-13)
    assert_parity(mon, exp_mon, tol=1e-13)


def test_free_function_until_single_and_all(torch_cuda, oracle):
    from tests import capi

    L = capi.lib()
    e = lattices.fodo_ring()
    lat = e.cbuffer.to_image()
    be = capi.c_buffer_from_image(lat)
    q = lattices.gaussian_particles(256, seed=31)
    blk = q.block.copy()
    sp = capi.particles_view(blk)
    assert L.st_Track_all_particles_until_turn(C.byref(sp), be, 7) == 0, _err()
    exp = q.block.copy()
    oracle.track_until(lat, exp, 7)
    assert_parity(blk, exp, tol=1e-13)
    blk2 = q.block.copy()
    sp2 = capi.particles_view(blk2)
    assert L.st_Track_particle_until_turn(C.byref(sp2), 5, be, 7) == 0
    exp2 = q.block.copy()
    oracle.track_until(lat, exp2, 7, i0=5, i1=6)
    assert_parity(blk2, exp2, tol=1e-13)
    L.st_Buffer_delete(be)


def test_trackjobnew_c_abi(torch_cuda, oracle):
    """The TrackJobNew entry points (track/track_job_base.h) on one job:
    construction with output, accessors, tracking, collect and reset."""
    import ctypes as Cc

    from sixtracklib_gb300 import ParticlesSet, _native

    L = _native.load()
    vp, u64, cb, u16 = Cc.c_void_p, Cc.c_uint64, Cc.c_bool, Cc.c_uint16
    sig = {"st_TrackJobNew_new_with_output": ([Cc.c_char_p, vp, vp, vp, u64, Cc.c_char_p], vp),
           "st_TrackJobNew_owns_output_buffer": ([vp], cb),
           "st_TrackJobNew_has_output_buffer": ([vp], cb),
           "st_TrackJobNew_has_beam_monitors": ([vp], cb),
           "st_TrackJobNew_get_num_beam_monitors": ([vp], u64),
           "st_TrackJobNew_get_total_num_of_particles": ([vp], u64),
           "st_TrackJobNew_get_arch_string": ([vp], Cc.c_char_p),
           "st_TrackJobNew_get_particles_buffer": ([vp], vp),
           "st_TrackJobNew_get_collect_flags": ([vp], u16),
           "st_TrackJobNew_track_until": ([vp, u64], Cc.c_int32),
           "st_TrackJobNew_collect_particles": ([vp], Cc.c_int32),
           "st_TrackJobNew_reset": ([vp, vp, vp, vp], Cc.c_int32),
           "st_TrackJobNew_delete": ([vp], None)}
    for name, (args, res) in sig.items():
        getattr(L, name).argtypes = args
        getattr(L, name).restype = res
    e = lattices.fodo_ring()
    e.BeamMonitor(num_stores=4, start=0, skip=1, is_rolling=1, is_turn_ordered=1)
    ps = ParticlesSet()
    p = ps.Particles(num_particles=100)
    q = lattices.gaussian_particles(100, seed=15)
    p.set_block(q.block)
    from tests import capi

    pb = capi.c_buffer_from_image(ps.cbuffer.to_image())
    eb = capi.c_buffer_from_image(e.cbuffer.to_image())
    job = L.st_TrackJobNew_new_with_output(b"cuda", pb, eb, None, 0, b"mode=exact")
    assert job, _native.last_error()
    assert L.st_TrackJobNew_has_output_buffer(job) and L.st_TrackJobNew_owns_output_buffer(job)
    assert L.st_TrackJobNew_has_beam_monitors(job)
    assert L.st_TrackJobNew_get_num_beam_monitors(job) == 1
    assert L.st_TrackJobNew_get_total_num_of_particles(job) == 100
    assert L.st_TrackJobNew_get_arch_string(job) == b"cuda"
    assert L.st_TrackJobNew_get_particles_buffer(job) == pb
    assert L.st_TrackJobNew_track_until(job, 10) == 0
    assert L.st_TrackJobNew_collect_particles(job) == 0
    got = capi_columns(pb)
    exp = q.block.copy()
    oracle.track_until(e.cbuffer.to_image(), exp, 10)
    assert_parity(got, exp, tol=1e-13)
    # reset on fresh particles: tracking starts over
    pb2 = capi.c_buffer_from_image(ps.cbuffer.to_image())
    assert L.st_TrackJobNew_reset(job, pb2, eb, None) == 0
    assert L.st_TrackJobNew_track_until(job, 3) == 0
    assert L.st_TrackJobNew_collect_particles(job) == 0
    exp3 = q.block.copy()
    oracle.track_until(e.cbuffer.to_image(), exp3, 3)
    assert_parity(capi_columns(pb2), exp3, tol=1e-13)
    L.st_TrackJobNew_delete(job)
    for b in (pb, pb2, eb):
        L.st_Buffer_delete(b)


def test_trackjobnew_debug_mode_c_abi(torch_cuda, oracle):
    """st_TrackJobNew_{is_in,enable,disable}_debug_mode and the debug
    register (track/track_job_base.h:182-189, track/track_kernel_impl.h:
    149-250): in debug mode a valid call tracks as in normal mode and leaves
    the track status in the register's low bits; invalid line boundaries and
    an elem-by-elem call without an output raise their flags and return -1
    without tracking; out of debug mode the same calls fail as before."""
    import ctypes as Cc

    from sixtracklib_gb300 import ParticlesSet, _native
    from tests import capi

    L = _native.load()
    vp, u64, cb = Cc.c_void_p, Cc.c_uint64, Cc.c_bool
    sig = {"st_TrackJobNew_new": ([Cc.c_char_p, vp, vp, Cc.c_char_p], vp),
           "st_TrackJobNew_is_in_debug_mode": ([vp], cb),
           "st_TrackJobNew_enable_debug_mode": ([vp], Cc.c_int32),
           "st_TrackJobNew_disable_debug_mode": ([vp], Cc.c_int32),
           "st_TrackJobNew_collect_debug_flag": ([vp], Cc.c_int32),
           "st_TrackJobNew_get_debug_register": ([vp], u64),
           "st_TrackJobNew_track_until": ([vp, u64], Cc.c_int32),
           "st_TrackJobNew_track_line": ([vp, u64, u64, cb], Cc.c_int32),
           "st_TrackJobNew_track_elem_by_elem": ([vp, u64], Cc.c_int32),
           "st_TrackJobNew_collect_particles": ([vp], Cc.c_int32),
           "st_TrackJobNew_delete": ([vp], None)}
    for name, (args, res) in sig.items():
        getattr(L, name).argtypes = args
        getattr(L, name).restype = res
    e = lattices.fodo_ring()
    n_elem = len(e)
    ps = ParticlesSet()
    p = ps.Particles(num_particles=200)
    q = lattices.gaussian_particles(200, seed=17, sx=5e-3, sy=5e-3)
    p.set_block(q.block)
    pb = capi.c_buffer_from_image(ps.cbuffer.to_image())
    eb = capi.c_buffer_from_image(e.cbuffer.to_image())
    job = L.st_TrackJobNew_new(b"cuda", pb, eb, b"mode=exact")
    assert job, _native.last_error()
    assert not L.st_TrackJobNew_is_in_debug_mode(job)
    assert L.st_TrackJobNew_collect_debug_flag(job) == -1
    assert L.st_TrackJobNew_enable_debug_mode(job) == 0
    assert L.st_TrackJobNew_is_in_debug_mode(job)
    assert L.st_TrackJobNew_collect_debug_flag(job) == 0
    # a valid call: tracks, the register holds status 0 and no flag
    assert L.st_TrackJobNew_track_until(job, 20) == 0
    assert L.st_TrackJobNew_get_debug_register(job) == 0
    assert L.st_TrackJobNew_collect_particles(job) == 0
    exp = q.block.copy()
    oracle.track_until(e.cbuffer.to_image(), exp, 20)
    assert_parity(capi_columns(pb), exp, tol=1e-13)
    # invalid line boundaries: flag 2^39, -1, nothing tracked
    before = capi_columns(pb).copy()
    assert L.st_TrackJobNew_track_line(job, 5, n_elem + 3, False) == -1
    reg = L.st_TrackJobNew_get_debug_register(job)
    assert reg & (1 << 39) and (reg & 0xFFFFFFFF) == 0xFFFFFFFF
    assert L.st_TrackJobNew_collect_particles(job) == 0
    assert np.array_equal(capi_columns(pb), before)
    # elem-by-elem without an output: the engine's flag 2^42
    assert L.st_TrackJobNew_track_elem_by_elem(job, 21) == -1
    assert L.st_TrackJobNew_get_debug_register(job) & (1 << 42)
    # a valid line call afterwards clears the register
    assert L.st_TrackJobNew_track_line(job, 0, 10, False) == 0
    assert L.st_TrackJobNew_get_debug_register(job) == 0
    # out of debug mode: the invalid line is refused as before
    assert L.st_TrackJobNew_disable_debug_mode(job) == 0
    assert not L.st_TrackJobNew_is_in_debug_mode(job)
    assert L.st_TrackJobNew_track_line(job, 5, n_elem + 3, False) == -1
    assert "line range" in _native.last_error()
    assert L.st_TrackJobNew_enable_debug_mode(None) == -1
    L.st_TrackJobNew_delete(job)
    for b in (pb, eb):
        L.st_Buffer_delete(b)


def capi_columns(c_buffer):
    """The 21 x n columns of Particles object 0 of a C-side buffer."""
    from sixtracklib_gb300.trackjob import _c_columns
    from sixtracklib_gb300 import _native

    return _c_columns(_native.load(), c_buffer, 0)


def test_trackjob_monitor_output_into_stored_buffer(torch_cuda):
    """A BeamMonitor whose out_address is assigned from a particle set in a
    stored buffer (tests/python/test_track_job_cpu_assign_address_items.py):
    after tracking, collect_stored_buffer leaves the monitor's turn-by-turn
    records there, equal to the job's own monitor output."""
    from sixtracklib_gb300 import ParticlesSet
    from sixtracklib_gb300.beam_elements import TYPE_BEAM_MONITOR
    from sixtracklib_gb300.particles import TYPE_PARTICLE
    from sixtracklib_gb300.trackjob import TrackJob

    e = lattices.fodo_ring()
    bm = len(e)
    e.BeamMonitor(num_stores=4, start=0, skip=1, is_rolling=0, is_turn_ordered=1)
    ps = ParticlesSet()
    p = ps.Particles(num_particles=64)
    p.set_block(lattices.gaussian_particles(64, seed=19).block)
    out = ParticlesSet()
    out.Particles(num_particles=4 * 64)
    job = TrackJob(e, ps, config_str="mode=exact")
    oid = job.add_stored_buffer(cbuffer=out)
    assert job.stored_buffer(oid).num_objects == 1 and job.ptr_stored_buffer(oid)
    job.add_assign_address_item(
        dest_elem_type_id=TYPE_BEAM_MONITOR, dest_buffer_id=2, dest_elem_index=bm,
        dest_pointer_offset=24, src_elem_type_id=TYPE_PARTICLE, src_buffer_id=oid,
        src_elem_index=0, src_pointer_offset=0)
    job.commit_address_assignments()
    job.assign_all_addresses()
    assert e.get(bm).out_address != 0
    job.track_until(4)
    job.collect_stored_buffer(oid)
    job.collect_output()
    mon = job.output_particles(job.beam_monitor_output_offset)
    got = out.particles[0]
    assert np.array_equal(got.block, mon.block)
    assert np.count_nonzero(got.x) > 200 and set(np.unique(got.at_turn)) == {0, 1, 2, 3}


def test_cuda_trackjob_properties_and_track_line(torch_cuda, oracle):
    """CudaTrackJob as the reference's CUDA tests drive it
    (tests/python/cuda/test_track_job_threads_per_block.py,
    test_track_job_track_line.py): particle-set index as the third
    argument, dotted TOML keys, the job's properties, and tracking line by
    line, element after element, until a full turn."""
    from sixtracklib_gb300 import ParticlesSet
    from sixtracklib_gb300.trackjob import CudaTrackJob

    e = lattices.fodo_ring()
    ps = ParticlesSet()
    ps.Particles(num_particles=10)  # set 0: not tracked
    p = ps.Particles(num_particles=200)
    q = lattices.gaussian_particles(200, seed=23)
    p.set_block(q.block)
    cfg = "cuda.threads_per_block = 256\r\ncuda.track_threads_per_block = 512\r\n"
    job = CudaTrackJob(e, ps, 1, config_str=cfg)
    assert job.arch_str == "cuda" and job.is_collecting_particles and job.requires_collecting
    assert job.has_controller and job.has_particles_arg and job.has_beam_elements_arg
    assert not job.is_in_debug_mode and not job.has_output_buffer and not job.owns_output_buffer
    assert job.num_particle_sets == 1
    assert job.type() == job.arch_id == 3  # SIXTRL_ARCHITECTURE_CUDA
    assert CudaTrackJob.enabled_archs() == ["cuda"]
    assert CudaTrackJob.num_available_nodes("cuda") >= 1
    assert CudaTrackJob.num_available_nodes("opencl") == 0
    assert job.default_threads_per_block == 256
    assert job.default_track_threads_per_block == 256  # 512 requested: the kernel's maximum
    n = len(e)
    for k in range(n):
        job.track_line(k, k + 1, finish_turn=(k == n - 1))
        assert job.last_track_status_success
    job.collect_particles()
    exp = q.block.copy()
    oracle.track_until(e.cbuffer.to_image(), exp, 1)
    got = ps.particles[1].block.copy()
    assert_parity(got, exp, tol=1e-13)
    assert np.all(got[19].view(np.int64) == 1) and np.all(got[18].view(np.int64) == 0)
    np.testing.assert_array_equal(ps.particles[0].x, 0.0)  # the other set is untouched
    with pytest.raises(RuntimeError):
        CudaTrackJob(e, ps, 0, config_str="cuda.threads_per_block = 48")


def test_trackjob_particle_addresses(torch_cuda, oracle):
    """Device addresses of the job's particle columns
    (tests/python/cuda/test_track_job_fetch_particle_addr.py): consistent
    with the column layout, and usable in place -- tracking the fetched
    block with the device-resident entry point changes what the job
    collects."""
    from sixtracklib_gb300 import ParticlesSet, _native
    from sixtracklib_gb300.device import DeviceTracker
    from sixtracklib_gb300.trackjob import CudaTrackJob

    e = lattices.fodo_ring()
    ps = ParticlesSet()
    p = ps.Particles(num_particles=300)
    q = lattices.gaussian_particles(300, seed=27)
    p.set_block(q.block)
    job = CudaTrackJob(e, ps, 0, config_str="mode=exact")
    assert job.can_fetch_particle_addresses and not job.has_particle_addresses
    assert job.get_particle_addresses(0) is None
    job.fetch_particle_addresses()
    assert job.last_status_success and job.has_particle_addresses
    a = job.get_particle_addresses(0)
    assert a.num_particles == 300 and job.get_particle_addresses(1) is None
    cols = [getattr(a, f) for f, _ in a._fields_[1:]]
    assert all(c2 - c1 == 300 * 8 for c1, c2 in zip(cols, cols[1:]))
    job.track_until(2)
    trk = DeviceTracker(e, config="mode=exact")
    lib = _native.load()
    assert lib.st_DeviceLattice_track_until(trk._ptr, C.c_void_p(a.q0), 300, 5, None) == 0
    torch_cuda.cuda.synchronize()
    job.collect_particles()
    exp = q.block.copy()
    oracle.track_until(e.cbuffer.to_image(), exp, 5)
    assert_parity(ps.particles[0].block.copy(), exp, tol=1e-13)
    job.clear_particle_addresses(0)
    assert not job.has_particle_addresses and job.get_particle_addresses(0) is None


class _StAssignItem(C.Structure):
    _fields_ = [(n, C.c_uint64) for n in (
        "dest_buffer_id", "src_buffer_id", "dest_elem_type_id", "src_elem_type_id",
        "dest_elem_index", "src_elem_index", "dest_pointer_offset", "src_pointer_offset")]


def _c_image(lib, ptr):
    n = lib.st_Buffer_get_size(ptr)
    data = lib.st_Buffer_get_const_data_begin(ptr)
    return np.ctypeslib.as_array(C.cast(data, C.POINTER(C.c_uint64)), shape=(n // 8,)).copy()


def test_c_trackjob_stored_buffers_and_address_assignment(torch_cuda, oracle):
    """The C functions for stored buffers and assignment items
    (common/track_job.h, NS(TrackJob_add_stored_buffer) ...
    NS(TrackJob_assign_all_addresses)) on one C TrackJob: ids and
    ownership, item bookkeeping, line-density tables assigned from a stored
    buffer to interpolated space-charge kicks (tracked result equal to the
    oracle on the job's lattice, different from the fallback density),
    refused items, and a BeamMonitor writing into a stored particle set."""
    from sixtracklib_gb300 import ParticlesSet, _native
    from sixtracklib_gb300.beam_elements import (TYPE_BEAM_MONITOR, TYPE_LINE_DENSITY_PROF_DATA,
                                                 TYPE_SC_INTERPOLATED_PROF)
    from sixtracklib_gb300.particles import TYPE_PARTICLE
    from tests import capi

    L = _native.load()
    z = np.linspace(-0.3, 0.3, 41)
    prof = np.exp(-0.5 * (z / 0.1) ** 2) * 1e12
    tables = Elements()
    tables.LineDensityProfileData(values=prof, z0=-0.3, dz=float(z[1] - z[0]), method="linear")
    tables.LineDensityProfileData(values=prof * 1.1, z0=-0.3, dz=float(z[1] - z[0]),
                                  method="cubic")
    e = lattices.fodo_ring()
    first = len(e)
    for k in range(6):
        e.SCInterpolatedProfile(number_of_particles=1e11, length=0.5, sigma_x=1e-3,
                                sigma_y=1.2e-3 if k % 2 else 1e-3, interpol_data_addr=0,
                                line_density_prof_fallback=5e11, min_sigma_diff=1e-10)
    ps = ParticlesSet()
    p = ps.Particles(num_particles=256)
    q = lattices.gaussian_particles(256, seed=31, sz=0.12)
    p.set_block(q.block)
    pb = capi.c_buffer_from_image(ps.cbuffer.to_image())
    eb = capi.c_buffer_from_image(e.cbuffer.to_image())
    sb = capi.c_buffer_from_image(tables.cbuffer.to_image())
    idx = (C.c_uint64 * 1)(0)
    job = L.st_TrackJob_new_detailed(b"cuda", pb, 1, idx, eb, None, 0, b"mode=exact")
    assert job, _native.last_error()

    assert not L.st_TrackJob_has_stored_buffers(job) and L.st_TrackJob_min_stored_buffer_id(job) == 0
    bid = L.st_TrackJob_add_stored_buffer(job, sb, False, False)
    assert bid == 1024 and L.st_TrackJob_create_stored_buffer(job, 256) == 1025
    assert L.st_TrackJob_owns_stored_buffer(job, 1025) and not L.st_TrackJob_owns_stored_buffer(job, 1024)
    assert L.st_TrackJob_stored_buffer(job, 1024) == sb and L.st_TrackJob_num_stored_buffers(job) == 2
    assert L.st_TrackJob_remove_stored_buffer(job, 1025) == 0
    assert L.st_TrackJob_remove_stored_buffer(job, 1025) == -1
    # taking ownership without deleting: the contents move, the caller's buffer is empty
    moved = capi.c_buffer_from_image(tables.cbuffer.to_image())
    first_obj = int(C.cast(L.st_Buffer_get_const_object(moved, 0), C.POINTER(C.c_uint64))[0])
    mid = L.st_TrackJob_add_stored_buffer(job, moved, True, False)
    kept = L.st_TrackJob_stored_buffer(job, mid)
    assert mid == 1026 and kept != moved and L.st_Buffer_get_num_of_objects(moved) == 0
    assert int(C.cast(L.st_Buffer_get_const_object(kept, 0), C.POINTER(C.c_uint64))[0]) == first_obj
    L.st_Buffer_delete(moved)
    assert L.st_TrackJob_remove_stored_buffer(job, mid) == 0
    assert (L.st_TrackJob_min_stored_buffer_id(job), L.st_TrackJob_max_stored_buffer_id(job)) == (1024, 1024)

    ptrs = [L.st_TrackJob_add_assign_address_item_detailed(
        job, TYPE_SC_INTERPOLATED_PROF, 2, first + k, 48, TYPE_LINE_DENSITY_PROF_DATA, bid, k % 2, 0)
        for k in range(6)]
    assert all(ptrs)
    again = _StAssignItem(2, bid, TYPE_SC_INTERPOLATED_PROF, TYPE_LINE_DENSITY_PROF_DATA,
                          first + 3, 1, 48, 0)
    assert L.st_TrackJob_add_assign_address_item(job, C.byref(again)) == ptrs[3]
    assert L.st_TrackJob_total_num_assign_items(job) == 6
    assert L.st_TrackJob_num_assign_items(job, 2, bid) == 6 and L.st_TrackJob_has_assign_items(job, 2, bid)
    assert not L.st_TrackJob_has_assign_items(job, 2, 1)
    assert L.st_TrackJob_has_assign_item_by_index(job, 2, bid, 5)
    assert not L.st_TrackJob_has_assign_item_by_index(job, 2, bid, 6)
    assert L.st_TrackJob_has_assign_address_item(job, C.byref(again))
    assert L.st_TrackJob_index_of_assign_address_item(job, C.byref(again)) == 3
    assert L.st_TrackJob_ptr_assign_address_item_by_index(job, 2, bid, 3) == ptrs[3]
    assert L.st_TrackJob_commit_address_assignments(job) == 0
    assert L.st_TrackJob_assign_all_addresses(job) == 0, _native.last_error()
    obj = C.cast(L.st_Buffer_get_const_object(sb, 1), C.POINTER(C.c_uint64))
    sc = C.cast(L.st_Buffer_get_const_object(eb, first + 3), C.POINTER(C.c_uint64))
    assert C.cast(sc[0] + 48, C.POINTER(C.c_uint64))[0] == obj[0]

    assert L.st_TrackJob_track_until(job, 5) == 0
    L.st_TrackJob_collect_particles(job)
    img = _c_image(L, eb)
    exp = q.block.copy()
    assert oracle.track_until(img, exp, 5) == 0
    assert_parity(capi_columns(pb), exp, tol=1e-13)
    fallback = q.block.copy()
    assert oracle.track_until(e.cbuffer.to_image(), fallback, 5) == 0
    assert not np.array_equal(exp, fallback)

    # an item whose source object does not exist is refused at commit and assignment
    L.st_TrackJob_add_assign_address_item_detailed(
        job, TYPE_SC_INTERPOLATED_PROF, 2, first, 48, TYPE_LINE_DENSITY_PROF_DATA, bid, 7, 0)
    assert L.st_TrackJob_commit_address_assignments(job) == -1
    assert L.st_TrackJob_assign_addresses(job, 2, bid) == -1
    L.st_TrackJob_delete(job)

    # a BeamMonitor writing into a particle set of a stored buffer
    e2 = lattices.fodo_ring()
    bm = len(e2)
    e2.BeamMonitor(num_stores=4, start=0, skip=1, is_rolling=0, is_turn_ordered=1)
    out = ParticlesSet()
    out.Particles(num_particles=4 * 256)
    pb2 = capi.c_buffer_from_image(ps.cbuffer.to_image())
    eb2 = capi.c_buffer_from_image(e2.cbuffer.to_image())
    ob = capi.c_buffer_from_image(out.cbuffer.to_image())
    job = L.st_TrackJob_new_detailed(b"cuda", pb2, 1, idx, eb2, None, 0, b"mode=exact")
    assert job, _native.last_error()
    oid = L.st_TrackJob_add_stored_buffer(job, ob, True, True)  # `ob` is deleted
    assert L.st_TrackJob_owns_stored_buffer(job, oid)
    ob = L.st_TrackJob_stored_buffer(job, oid)
    assert L.st_Buffer_get_num_of_objects(ob) == 1
    assert L.st_TrackJob_add_assign_address_item_detailed(
        job, TYPE_BEAM_MONITOR, 2, bm, 24, TYPE_PARTICLE, oid, 0, 0)
    assert L.st_TrackJob_assign_addresses(job, 2, oid) == 0, _native.last_error()
    assert L.st_TrackJob_track_until(job, 4) == 0
    assert L.st_TrackJob_collect_stored_buffer(job, oid) == 0
    got = capi_columns(ob)
    outb = L.st_TrackJob_get_output_buffer(job)
    off = L.st_TrackJob_get_beam_monitor_output_buffer_offset(job)
    from sixtracklib_gb300.trackjob import _c_columns

    mon = _c_columns(L, outb, off)
    assert np.array_equal(got, mon)
    assert set(np.unique(got[19].view(np.int64))) == {0, 1, 2, 3}  # at_turn
    assert np.count_nonzero(got[6]) > 800  # x
    L.st_TrackJob_delete(job)  # frees the owned stored buffer
    for b in (pb, eb, sb, pb2, eb2):
        L.st_Buffer_delete(b)


@pytest.mark.gpu
@pytest.mark.parametrize("aperture,min_length,limits", [
    ("always", 0.0, (1.0, 1.0)), ("conditional", 5.0, (1.0, 1.0)),
    ("conditional", 11.0, (1.0, 1.0)), ("never", 0.0, (1.0, 1.0)),
    ("always", 0.0, (0.5, 0.8))])
def test_global_aperture_over_drifts(torch_cuda, oracle, aperture, min_length, limits):
    """100 particles over 10,000 drifts of 10 m
    (common/test_particles_aperture_c99.cpp:30-122): with the global
    aperture checked after a drift, a particle is lost exactly at the first
    drift that takes |x| or |y| beyond the limit, and never otherwise; the
    same for the conditional check (drifts at least `aperture_min_length`
    long) and custom limits.  Bit-identical to the oracle set up alike."""
    from sixtracklib_gb300.device import DeviceTracker

    e = Elements()
    for _ in range(10_000):
        e.Drift(length=10.0)
    rng = np.random.default_rng(30)
    p = lattices.gaussian_particles(100, seed=30)
    p.x[:], p.y[:] = rng.normal(0, 1e-3, 100), rng.normal(0, 1e-3, 100)
    p.px[:], p.py[:] = rng.uniform(-2e-5, 2e-5, 100), rng.uniform(-1.5e-5, 1.5e-5, 100)
    lat = e.cbuffer.to_image()
    xl, yl = limits
    mode = {"always": 2, "conditional": 1, "never": 0}[aperture]
    oracle.set_aperture_mode(mode, min_length, xl, yl)
    try:
        exp = p.block.copy()
        s0 = oracle.track_until(lat, exp, 1)
    finally:
        oracle.set_aperture_mode()
    trk = DeviceTracker(lat, config=f"mode=exact aperture={aperture} "
                                    f"aperture_min_length={min_length} x_limit={xl} y_limit={yl}")
    cols = torch_cuda.from_numpy(p.block.copy().view(np.int64)).cuda()
    st = trk.track_until(cols, 1)
    torch_cuda.cuda.synchronize()
    got = cols.cpu().numpy().view(np.uint64)
    assert st == s0 == 0
    assert_parity(got, exp, 0.0, bit_exact=True)
    state = got[20].view(np.int64)
    checked = mode == 2 or (mode == 1 and 10.0 >= min_length)
    if not checked:
        assert np.all(state == 1)
        return
    lost = state == 0
    assert 10 < lost.sum() < 100
    x, y = got[6].view(np.float64), got[7].view(np.float64)
    px, py = p.px * p.rpp, p.py * p.rpp
    # lost particles keep the coordinates past the limit at their drift
    assert np.all((np.abs(x[lost]) > xl) | (np.abs(y[lost]) > yl))
    assert np.all((np.abs(x[~lost]) <= xl) & (np.abs(y[~lost]) <= yl))
    # ... and the first drift to cross it, from the straight-line orbit
    k = got[18].view(np.int64)[lost]
    x0, y0 = p.x[lost], p.y[lost]
    before = (k * 10.0)
    assert np.all((np.abs(x0 + px[lost] * before) <= xl * (1 + 1e-9)) &
                  (np.abs(y0 + py[lost] * before) <= yl * (1 + 1e-9)))


def test_segmented_long_call_bit_identical(torch_cuda, oracle):
    """A waiting until-turn call of many turns runs as capped launches with
    the surviving particles re-packed between them; the result equals one
    uncapped launch (launch_until) bit for bit, also with particles that
    start at different turns, and a strided sample agrees with the oracle."""
    torch = torch_cuda
    from sixtracklib_gb300.device import DeviceTracker

    e = lattices.synthetic_ring()
    trk = DeviceTracker(e, config="mode=fast")
    p = lattices.polar_grid_particles(300_000, seed=8)
    p.at_turn[::7] = 2  # mixed start turns
    base = torch.from_numpy(p.block.copy().view(np.int64)).cuda()
    a = base.clone()
    assert trk.track_until(a, 6) == 0  # 300k x 20k elements per turn: one turn per launch
    b = base.clone()
    trk.launch_until(b, 6)
    assert trk.last_status() == 0
    assert torch.equal(a, b)
    lost = int((a[20] == 0).sum())
    assert 0 < lost < 300_000
    idx = np.arange(0, 300_000, 293)[:1024]
    sample = p.block[:, idx].copy()
    assert oracle.track_until(e.cbuffer.to_image(), sample, 6) == 0
    # fast mode: within 1e-13 per turn, growing with the turns (1e-10 at 1000)
    assert_parity(a.cpu().numpy().view(np.uint64)[:, idx], sample, tol=1e-11)
