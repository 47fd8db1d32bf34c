"""The engine against the reference's own CUDA kernel on the same GPU
(sixtracklib/cuda/kernels/track_particles.cu compiled for sm_103a with the
reference's release flags, launched as its CUDA TrackJob launches it:
oracle/ref_cuda.py).  Both sides evaluate sin, exp and sqrt with CUDA's
libm, so the engine's exact mode reproduces the reference kernel bit for
bit on lattices of drifts, multipoles, cavities, shifts, rotations, edges
and apertures; the beam-field maps agree within the tolerance of the field
evaluation (the engine's Faddeeva function is a division-free form of the
same truncated expression).  Skipped where the cubin was not built (it needs
the reference sources)."""

import numpy as np
import pytest

from sixtracklib_gb300 import lattices
from sixtracklib_gb300.beam_elements import Elements
from tests.test_gpu_parity import assert_parity, run_device, torch_cuda  # noqa: F401

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ref_kernels(torch_cuda):
    from oracle import ref_cuda

    if not ref_cuda.available():
        pytest.skip("reference CUDA kernels not built (oracle/build_ref_cuda.sh)")
    return ref_cuda.RefCudaKernels(torch_cuda)


def _ref_until(k, torch, lat, block, turns):
    from oracle import ref_cuda

    d_lat = k.to_device(lat)
    d_p = k.to_device(ref_cuda.particles_image(block))
    k.track_until(d_p, block.shape[1], d_lat, turns)
    torch.cuda.synchronize()
    return ref_cuda.particles_block(d_p)


def _ref_line(k, torch, lat, block, begin, end, finish):
    from oracle import ref_cuda

    d_lat = k.to_device(lat)
    d_p = k.to_device(ref_cuda.particles_image(block))
    k.track_line(d_p, block.shape[1], d_lat, begin, end, finish)
    torch.cuda.synchronize()
    return ref_cuda.particles_block(d_p)


def test_fodo_ring_1000_turns_bit_identical(torch_cuda, ref_kernels):
    """The FODO ring with its cavity, 10,000 protons, 1,000 turns."""
    lat = lattices.fodo_ring().cbuffer.to_image()
    p = lattices.gaussian_particles(10_000, seed=2024)
    ref = _ref_until(ref_kernels, torch_cuda, lat, p.block, 1000)
    st, got = run_device(torch_cuda, lat, p.block, until=1000, mode="exact")
    assert st == 0
    assert_parity(got, ref, 0.0, bit_exact=True)


def test_synthetic_ring_bit_identical(torch_cuda, ref_kernels):
    """The 20,000-element ring (cavities included) on 16,384 particles of the
    polar grid, 3 turns, losses included."""
    lat = lattices.synthetic_ring().cbuffer.to_image()
    p = lattices.polar_grid_particles(16384, seed=12)
    ref = _ref_until(ref_kernels, torch_cuda, lat, p.block, 3)
    st, got = run_device(torch_cuda, lat, p.block, until=3, mode="exact")
    assert st == 0
    assert_parity(got, ref, 0.0, bit_exact=True)
    lost = int((ref[20].view(np.int64) == 0).sum())
    assert 0 < lost < 16384


def test_line_and_misc_elements_bit_identical(torch_cuda, ref_kernels):
    e = Elements()
    for _ in range(20):
        e.Drift(length=1.3)
        e.DriftExact(length=0.7)
        e.Multipole(knl=[1e-5, 0.01, 0.02, 0.3], ksl=[0.0, 1e-4], hxl=1e-6, length=1.0)
        e.SRotation(angle=3.0)
        e.XYShift(dx=1e-5, dy=-2e-5)
        e.DipoleEdge(r21=1e-3, r43=-1e-3)
        e.RFMultipole(voltage=1e4, frequency=4e8, lag=30.0, knl=[1e-6, 1e-5], ksl=[0.0, 2e-6],
                      pn=[0.0, 10.0], ps=[5.0, 0.0])
        e.Cavity(voltage=2e5, frequency=4e8, lag=170.0)
        e.Multipole(knl=[0.0, -0.01])
        e.LimitRectEllipse(max_x=0.02, max_y=0.015, a=0.025, b=0.02)
        e.LimitRect(min_x=-0.019, max_x=0.02, min_y=-0.02, max_y=0.014)
    lat = e.cbuffer.to_image()
    p = lattices.gaussian_particles(3000, seed=3, sx=4e-3, sy=4e-3, spx=1e-4, spy=1e-4)
    for begin, end, finish in ((0, len(e), True), (17, 93, False)):
        ref = _ref_line(ref_kernels, torch_cuda, lat, p.block, begin, end, finish)
        st, got = run_device(torch_cuda, lat, p.block, line=(begin, end, finish), mode="exact")
        assert st == 0
        assert_parity(got, ref, 0.0, bit_exact=True)
    ref = _ref_until(ref_kernels, torch_cuda, lat, p.block, 3)
    st, got = run_device(torch_cuda, lat, p.block, until=3, mode="exact")
    assert_parity(got, ref, 0.0, bit_exact=True)
    lost = int((ref[20].view(np.int64) == 0).sum())
    assert 0 < lost < 3000


@pytest.mark.parametrize("elliptic", [False, True])
def test_beam_beam_space_charge(torch_cuda, ref_kernels, elliptic):
    """FODO ring + 4 BB6D (21 slices) + 4 BB4D + 200 q-Gaussian kicks:
    1e-13 after one turn, 1e-10 after 20, loss flags and counters identical."""
    lat = lattices.bb_sc_ring(elliptic=elliptic).cbuffer.to_image()
    p = lattices.gaussian_particles(1024, seed=17, sx=2e-5, sy=2e-5)
    for turns, tol in ((1, 1e-13), (20, 1e-10)):
        ref = _ref_until(ref_kernels, torch_cuda, lat, p.block, turns)
        for mode in ("exact", "fast"):
            st, got = run_device(torch_cuda, lat, p.block, until=turns, mode=mode)
            assert st == 0
            assert_parity(got, ref, tol=tol)


def test_benchmark_workload_full_size_bit_identical(torch_cuda, ref_kernels):
    """The benchmark workload at full size -- 1,000,000 protons of the polar
    grid on the 20,000-element ring, 2 turns -- tracked by the reference's
    kernel and by the engine's exact mode: every column of every particle
    bit-identical, losses included."""
    from sixtracklib_gb300.device import DeviceTracker

    torch = torch_cuda
    e = lattices.synthetic_ring()
    p = lattices.polar_grid_particles(1_000_000)
    ref = _ref_until(ref_kernels, torch, e.cbuffer.to_image(), p.block, 2)
    trk = DeviceTracker(e, config="mode=exact")
    cols = torch.from_numpy(p.block.copy().view(np.int64)).cuda()
    assert trk.track_until(cols, 2) == 0
    got = cols.cpu().numpy().view(np.uint64)
    lost = int((ref[20].view(np.int64) == 0).sum())
    assert 0 < lost < 1_000_000
    diff = np.nonzero((got != ref).any(axis=1))[0]
    assert diff.size == 0, f"columns {diff} differ"
