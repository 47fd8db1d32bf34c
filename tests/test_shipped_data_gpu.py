"""GPU parity on the reference's own shipped data (tests/testdata of the
reference), through the C ABI.

* `bbsimple`: the pysixtrack element-by-element dump (2 particles, Drift,
  Multipole, Cavity, BeamBeam4D, BeamBeam6D) reproduced by
  st_Track_all_particles_element_by_element_until_turn: the record stored
  before element k equals dump state k, the final state equals the last dump
  state (reference test: common/test_track_c99.cpp:389-630).
* `lhc_no_bb` (18,657 elements) and `beambeam` (10,866 elements, with the
  pysixtrack-initialised BeamBeam6D elements): 1,024 protons tracked by the
  reference build (tests/golden/ref_shipped_*.npz), 1 turn through the free
  function st_Track_all_particles_until_turn with host buffers and 1,000
  turns device-resident (st_DeviceLattice_track_until).

Tolerances are the reference's own: 1e-13 absolute for the LHC lattice
(common/test_track_c99.cpp:400) and 1e-14 absolute GPU against CPU
(cuda/track/test_track_job_track_until_c99.cpp:40) after one turn; 1e-10
absolute after 1,000 turns.  Integer columns (particle id, at_element,
at_turn, state) identical.  Beside the absolute deviation each test prints
the per-particle deviation normalised by that particle's own phase-space
amplitude (amplitude_dev: median, 99th percentile, maximum) and bounds the
maximum by 2e-9 after one turn and 2e-7 after 1,000 (measured on GB300:
exact mode 0 on lhc_no_bb, where only drifts, multipoles, shifts, rotations
and 12 cavities act, and 6e-11 / 2.2e-8 on beambeam, where CUDA's and the
host's exp differ in the last bit inside the beam-beam kicks; fast mode
5e-10 / 4e-9 and 6e-11 / 2.8e-8, medians 1e-12 to 5e-10).
"""

import ctypes as C
import os

import numpy as np
import pytest

from .deviation import amplitude_dev

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
COORDS = {"x": 6, "y": 7, "px": 8, "py": 9, "zeta": 10, "delta": 12}
REAL_COLS = [5, 6, 7, 8, 9, 10, 11, 12, 13, 14]  # s x y px py zeta psigma delta rpp rvv


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("GPU tests need a CUDA device")
    return torch


def load(name):
    return np.load(os.path.join(GOLDEN, name))


def f64(block, col):
    return block[col].view(np.float64)


def abs_dev(got, exp, cols=REAL_COLS):
    return max(float(np.max(np.abs(f64(got, c) - f64(exp, c)))) for c in cols)


def set_mode(monkeypatch, mode):
    monkeypatch.setenv("SIXTRACKLIB_GB300_CONFIG", f"mode={mode}")


@pytest.mark.parametrize("mode", ["exact", "fast"])
def test_bbsimple_pysixtrack_dump_elem_by_elem(torch_cuda, monkeypatch, mode):
    from sixtracklib_gb300 import _native
    from tests import capi

    set_mode(monkeypatch, mode)
    d = load("bbsimple.npz")
    lat, states = d["lattice"], d["states"]
    n_elem, npart = states.shape[0] - 1, states.shape[2]
    blk = states[0].copy()
    blk[20] = 1  # the dump marks state only on its last record
    pids = blk[17].view(np.int64)
    lo, hi = int(pids.min()), int(pids.max())
    nst = hi - lo + 1
    L = capi.lib()
    be = capi.c_buffer_from_image(lat)
    sp = capi.particles_view(blk)
    cfg = capi.StElemByElemConfig(0, nst, n_elem, 1, lo, 0, 0, hi, n_elem - 1, 0, 0, 0)
    out = np.zeros((21, nst * n_elem), dtype=np.uint64)
    ga = capi.generic_addr(out)
    cfg.out_store_addr = C.addressof(ga)
    st = L.st_Track_all_particles_element_by_element_until_turn(C.byref(sp), C.byref(cfg), be, 1)
    L.st_Buffer_delete(be)
    assert st == 0, _native.last_error()
    cols = [COORDS[k] for k in ("x", "y", "px", "py", "zeta", "delta")]
    worst = 0.0
    for k in range(n_elem):
        rec = out[:, k * nst + (pids - lo)]
        assert np.array_equal(rec[18].view(np.int64), np.full(npart, k)), "at_element of record"
        assert np.array_equal(rec[19].view(np.int64), np.zeros(npart, np.int64))
        worst = max(worst, abs_dev(rec, states[k], cols))
    # the final state: one turn done, at_element back to 0
    assert np.array_equal(blk[17:], states[-1][17:])
    worst = max(worst, abs_dev(blk, states[-1], cols))
    print(f"bbsimple {mode}: max |GPU - pysixtrack dump| = {worst:.2e}")
    assert worst <= 1e-14, worst


def _track_host(L, img, blk, turns):
    from sixtracklib_gb300 import _native
    from tests import capi

    be = capi.c_buffer_from_image(img)
    sp = capi.particles_view(blk)
    fn = L.st_Track_all_particles_until_turn
    fn.argtypes = [C.c_void_p, C.c_void_p, C.c_int64]
    fn.restype = C.c_int32
    st = fn(C.byref(sp), be, turns)
    L.st_Buffer_delete(be)
    return st, _native.last_error()


@pytest.mark.parametrize("mode", ["exact", "fast"])
@pytest.mark.parametrize("name", ["lhc_no_bb", "beambeam"])
def test_shipped_lattice_one_turn_host_buffers(torch_cuda, monkeypatch, name, mode):
    from tests import capi

    set_mode(monkeypatch, mode)
    d = load(f"ref_shipped_{name}.npz")
    blk = d["initial"].copy()
    st, err = _track_host(capi.lib(), d["lattice"], blk, 1)
    assert st == int(d["status_1"]), err
    exp = d["final_1"]
    assert np.array_equal(blk[17:], exp[17:]), "particle ids / at_element / at_turn / state"
    dev, (amed, a99, amax) = abs_dev(blk, exp), amplitude_dev(blk, exp, d["initial"])
    print(f"{name} {mode} 1 turn: abs {dev:.2e}; amplitude-normalised median {amed:.2e}, "
          f"99% {a99:.2e}, max {amax:.2e}")
    assert dev <= 1e-14, dev
    assert amax <= 2e-9, amax


@pytest.mark.parametrize("mode", ["exact", "fast"])
@pytest.mark.parametrize("name", ["lhc_no_bb", "beambeam"])
def test_shipped_lattice_1000_turns_device(torch_cuda, name, mode):
    from sixtracklib_gb300.device import DeviceTracker

    torch = torch_cuda
    d = load(f"ref_shipped_{name}.npz")
    trk = DeviceTracker(d["lattice"], config=f"mode={mode}")
    cols = torch.from_numpy(d["initial"].copy().view(np.int64)).cuda()
    st = trk.track_until(cols, 1000)
    torch.cuda.synchronize()
    got = cols.cpu().numpy().view(np.uint64)
    exp = d["final_1000"]
    assert st == int(d["status_1000"])
    assert np.array_equal(got[17:], exp[17:]), "particle ids / at_element / at_turn / state"
    dev, (amed, a99, amax) = abs_dev(got, exp), amplitude_dev(got, exp, d["initial"])
    print(f"{name} {mode} 1000 turns: abs {dev:.2e}; amplitude-normalised median {amed:.2e}, "
          f"99% {a99:.2e}, max {amax:.2e}")
    assert dev <= 1e-10, dev
    assert amax <= 2e-7, amax
