"""The TriCub map and the map feature flags on the GPU, through the C ABI,
against the reference's known-answer kicks and the reference builds'
outputs (tests/golden/, made by tests/golden/make_golden.py --tricub).

* exact mode: bit-identical to the reference's TriCub-enabled build (the
  per-cell coefficients computed on the GPU with the reference's arithmetic,
  the kick sums in its order);
* fast mode (Horner forms with FMAs): within 1e-13 of the column scale after
  one turn, 1e-10 after 20;
* the feature flags: the same status, losses and integer columns as the
  reference builds with the same flags, element by element and over whole
  turns; coordinates bit-identical except after the beam-beam and
  space-charge maps, whose exp / sqrt of CUDA's math library may differ from
  the host's in the last bit (1e-13 of the column scale there).
"""

import os

import numpy as np
import pytest

from . import tricub_cases as tc
from .test_gpu_parity import assert_parity, run_device, torch_cuda  # noqa: F401

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
ENABLED = "track_tricub=enabled"


def load(name):
    return np.load(os.path.join(GOLDEN, name))


def device(torch, lattice, block, config, until=None, line=None):
    from sixtracklib_gb300.device import DeviceTracker

    trk = DeviceTracker(lattice, config=config)
    cols = torch.from_numpy(block.copy().view(np.int64)).cuda()
    st = trk.track_line(cols, *line) if line is not None else trk.track_until(cols, until)
    torch.cuda.synchronize()
    return st, cols.cpu().numpy().view(np.uint64)


@pytest.mark.parametrize("mode", ["exact", "fast"])
def test_reference_known_answer_kicks(torch_cuda, mode):
    """tests/python/beam_elements/test_tricub.py:9-113: px, py, ptau after
    one TriCub of length 1 within np.allclose(rtol 1e-12, atol 1e-13)."""
    d = load("tricub_kicks.npz")
    e, p = tc.kicks_case(int(d["seed"]))
    st, got = device(torch_cuda, e.cbuffer.to_image(), p.block, f"mode={mode} {ENABLED}",
                     until=1)
    assert st == 0
    f = got.view(np.float64)
    np.testing.assert_allclose(np.stack([f[8], f[9], f[11] * f[2]], axis=1), d["kicks"],
                               rtol=1e-12, atol=1e-13)


@pytest.mark.parametrize("mode", ["exact", "fast"])
def test_tricub_ring_against_reference_build(torch_cuda, mode):
    d = load("ref_tricub.npz")
    for turns, tol in ((1, 1e-13), (20, 1e-10)):
        st, got = device(torch_cuda, d["lattice"], d["initial"], f"mode={mode} {ENABLED}",
                         until=turns)
        assert st == int(d[f"status_{turns}"]) == 0
        assert_parity(got, d[f"final_{turns}"], tol=tol, bit_exact=(mode == "exact"))


@pytest.mark.parametrize("build", list(tc.FLAG_BUILDS))
def test_feature_flags_against_reference_builds(torch_cuda, build):
    d = load("ref_flags.npz")
    img = d["lattice"]
    cfg = "mode=exact " + tc.flags_config(tc.FLAG_BUILDS[build])
    st, got = device(torch_cuda, img, d["initial"], cfg, until=3)
    assert st == int(d[f"until_status_{build}"])
    assert_parity(got, d[f"until_{build}"], tol=0.0, bit_exact=True)
    kinds = [type(o).__name__ for o in tc.flags_lattice().get_elements()]
    for k in range(d[f"line_{build}"].shape[0]):
        st, got = device(torch_cuda, img, d["initial"], cfg, line=(k, k + 1))
        assert st == int(d[f"line_status_{build}"][k]), k
        libm = kinds[k].startswith(("BeamBeam", "SC"))
        assert_parity(got, d[f"line_{build}"][k], tol=1e-13, bit_exact=not libm)


@pytest.mark.parametrize("mode", ["exact", "fast"])
def test_outside_the_grid_like_the_oracle(torch_cuda, oracle, mode):
    """Particles outside the grid fail the map and are lost there, as in
    the oracle (the reference reads outside its table)."""
    e, p = tc.kicks_case(5, n_part=300)
    p.x[::7] = -1.0
    p.zeta[3::11] = 5.0
    img = e.cbuffer.to_image()
    exp = p.block.copy()
    oracle.set_track_flags(2, 2, 2, 2)
    try:
        assert oracle.track_until(img, exp, 1) == -1
    finally:
        oracle.set_track_flags()
    st, got = device(torch_cuda, img, p.block, f"mode={mode} {ENABLED}", until=1)
    assert st == -1
    assert 40 < int((exp[20] == 0).sum()) < 100
    assert_parity(got, exp, tol=1e-13, bit_exact=(mode == "exact"))


def test_stored_buffer_assignment_like_the_reference_test(torch_cuda):
    """The reference's own flow (test_tricub.py, examples/python/tricub): the
    TriCubData in a stored buffer, its address assigned to the TriCub by the
    job; kicks as the in-lattice data gives them, and the known answer."""
    from sixtracklib_gb300 import TriCub_buffer_create_assign_address_item
    from sixtracklib_gb300.beam_elements import Elements
    from sixtracklib_gb300.particles import ParticlesSet
    from sixtracklib_gb300.trackjob import TrackJob

    d = load("tricub_kicks.npz")
    ref_e, ref_p = tc.kicks_case(int(d["seed"]))
    data = ref_e.cbuffer.get_object(1)
    lattice = Elements()
    lattice.TriCub(length=1.0)
    tables = Elements()
    tables.TriCubData(nx=data.nx, ny=data.ny, nz=data.nz, x0=data.x0, y0=data.y0, z0=data.z0,
                      dx=data.dx, dy=data.dy, dz=data.dz, table_addr=np.array(data.table_addr))
    ps = ParticlesSet()
    p = ps.Particles(num_particles=ref_p.num_particles)
    p.set_block(ref_p.block)
    job = TrackJob(lattice, ps, config_str=f"mode=exact {ENABLED}")
    bid = job.add_stored_buffer(cbuffer=tables)
    assert TriCub_buffer_create_assign_address_item(job, 0, bid, 0)
    job.commit_address_assignments()
    job.assign_all_addresses()
    assert job.track_until(1) == 0
    job.collect_particles()
    got = p.block.copy()
    st, exp = device(torch_cuda, ref_e.cbuffer.to_image(), ref_p.block, f"mode=exact {ENABLED}",
                     until=1)
    assert st == 0
    assert np.array_equal(got, exp)
    f = got.view(np.float64)
    np.testing.assert_allclose(np.stack([f[8], f[9], f[11] * f[2]], axis=1), d["kicks"],
                               rtol=1e-12, atol=1e-13)


def test_large_grid_and_shared_data(torch_cuda, oracle):
    """A 100 x 100 x 100 grid (the reference example's size; 970,299 cells,
    497 MB of coefficients computed on the GPU) used by two TriCub elements,
    and a small one: exact mode bit-identical to the oracle on a sample."""
    from sixtracklib_gb300 import lattices
    from sixtracklib_gb300.beam_elements import Elements

    rng = np.random.default_rng(12)
    e = Elements()
    e.TriCub(data=3, length=0.5, x_shift=1e-4)
    e.Drift(length=0.3)
    e.TriCub(data=4, length=0.7)
    n = 100
    e.TriCubData(nx=n, ny=n, nz=n, x0=-0.05, y0=-0.05, z0=-0.5, dx=1e-3, dy=1e-3, dz=1e-2,
                 table_addr=rng.uniform(-1, 1, n * n * n * 8) * 1e-12)
    e.TriCubData(nx=4, ny=4, nz=4, x0=-0.05, y0=-0.05, z0=-1.0, dx=0.04, dy=0.04, dz=0.7,
                 table_addr=rng.uniform(-1, 1, 4 * 4 * 4 * 8) * 1e-10)
    e.TriCub(data=3, length=0.2, y_shift=-2e-4)
    img = e.cbuffer.to_image()
    p = lattices.gaussian_particles(4096, seed=13, sx=5e-3, sy=5e-3, sz=0.1)
    exp = p.block.copy()
    oracle.set_track_flags(2, 2, 2, 2)
    try:
        assert oracle.track_until(img, exp, 3) == 0
    finally:
        oracle.set_track_flags()
    st, got = device(torch_cuda, img, p.block, f"mode=exact {ENABLED}", until=3)
    assert st == 0
    assert_parity(got, exp, tol=0.0, bit_exact=True)


def test_adjoint_refuses_tricub(torch_cuda):
    """The TriCub map has no adjoint: a differentiable call on a lattice with
    an enabled TriCub is refused before launch; skipped, the element is a
    no-op and the call runs."""
    from sixtracklib_gb300 import lattices
    from sixtracklib_gb300.autodiff import DifferentiableLattice

    ring, params = lattices.learnable_fodo_ring()
    n = len(ring)
    ring.TriCub(data=n + 1, length=0.5)
    ring.TriCubData(nx=4, ny=4, nz=4, x0=-0.1, y0=-0.1, z0=-2.0, dx=0.1, dy=0.1, dz=2.0)
    start = torch_cuda.from_numpy(lattices.gaussian_particles(256, seed=2).block.copy()
                                  .view(np.int64)).cuda()
    for flag, ok in (("enabled", False), ("skip", True)):
        lat = DifferentiableLattice(ring, params[:4], f"mode=exact track_tricub={flag}")
        end = start.clone()
        assert lat.tracker.track_until(end, 2) == 0
        lam = torch_cuda.ones((6, start.shape[1]), dtype=torch_cuda.float64, device="cuda")
        grad = torch_cuda.zeros(lat.num_params, dtype=torch_cuda.float64, device="cuda")
        if ok:
            lat.adjoint_turns(start, end, lam, 0, 2, grad)
        else:
            with pytest.raises(RuntimeError, match="TriCub"):
                lat.adjoint_turns(start, end, lam, 0, 2, grad)
