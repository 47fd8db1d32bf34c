"""Calls that overlap on one GPU through the asynchronous entry points.

st_DeviceLattice_launch_until returns before its kernel finishes.  The
particle-selection scratch and the status words it uses are shared by every
call on the GPU, so a second call launched on another stream must not
rewrite them while the first kernel still reads them: the engine orders the
second call's work after the first's on the GPU (an event per GPU).  Here a
long asynchronous launch on one stream is followed at once by a call with
more particles on another stream and another lattice, and by an adjoint
launch on a third; each result must equal the same call run alone.  The
caller's current device is unchanged by every call.
"""

import numpy as np
import pytest

from sixtracklib_gb300 import lattices

pytestmark = pytest.mark.gpu


def _torch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("GPU tests need a CUDA device")
    return torch


def test_overlapping_calls_on_two_streams_match_calls_alone():
    torch = _torch()
    from sixtracklib_gb300.device import DeviceTracker

    long_ring = DeviceTracker(lattices.synthetic_ring(), config="mode=fast")
    fodo = DeviceTracker(lattices.fodo_ring(), config="mode=fast")
    a0 = torch.from_numpy(lattices.polar_grid_particles(200_000, seed=5).block.copy()
                          .view(np.int64)).cuda()
    b0 = torch.from_numpy(lattices.gaussian_particles(400_000, seed=6, sx=6e-3, sy=6e-3)
                          .block.copy().view(np.int64)).cuda()
    # alone, one after the other
    a_ref, b_ref = a0.clone(), b0.clone()
    assert long_ring.track_until(a_ref, 2) == 0
    assert fodo.track_until(b_ref, 30) == 0
    torch.cuda.synchronize()
    # overlapping: the second call is issued while the first kernel runs
    dev_before = torch.cuda.current_device()
    a, b = a0.clone(), b0.clone()
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()
    torch.cuda.synchronize()
    with torch.cuda.stream(s1):
        long_ring.launch_until(a, 2)
    with torch.cuda.stream(s2):
        assert fodo.track_until(b, 30) == 0
    torch.cuda.synchronize()
    assert torch.cuda.current_device() == dev_before
    assert torch.equal(a, a_ref)
    assert torch.equal(b, b_ref)
    assert 0 < int((b[20] == 0).sum()) < b.shape[1]  # losses: the selection matters


def test_adjoint_after_async_launch_on_another_stream():
    torch = _torch()
    from sixtracklib_gb300.autodiff import DifferentiableLattice
    from sixtracklib_gb300.device import DeviceTracker

    ring, params = lattices.learnable_fodo_ring()
    lat = DifferentiableLattice(ring, params[:8], "mode=exact")
    start = torch.from_numpy(lattices.gaussian_particles(50_000, seed=9).block.copy()
                             .view(np.int64)).cuda()
    end = start.clone()
    assert lat.tracker.track_until(end, 3) == 0
    lam0 = torch.randn((6, start.shape[1]), dtype=torch.float64, device="cuda")

    def adjoint():
        lam = lam0.clone()
        grad = torch.zeros(lat.num_params, dtype=torch.float64, device="cuda")
        lat.adjoint_turns(start, end, lam, 0, 3, grad)
        return lam, grad

    lam_ref, grad_ref = adjoint()
    torch.cuda.synchronize()
    other = DeviceTracker(lattices.synthetic_ring(), config="mode=fast")
    busy = torch.from_numpy(lattices.polar_grid_particles(300_000, seed=2).block.copy()
                            .view(np.int64)).cuda()
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()
    torch.cuda.synchronize()
    with torch.cuda.stream(s1):
        other.launch_until(busy, 1)
    with torch.cuda.stream(s2):
        lam, grad = adjoint()
    torch.cuda.synchronize()
    assert other.last_status() == 0
    assert torch.equal(lam, lam_ref)
    torch.testing.assert_close(grad, grad_ref, rtol=1e-12, atol=0)  # atomics: order varies
