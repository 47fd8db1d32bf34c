"""The allocation-free until-turn entry point.

st_DeviceLattice_track_until_noalloc serves callers that must not allocate
device memory while they track (an operator inside a framework whose
buffers all come from the framework's own allocator, a loop with a fixed
memory budget): it keeps its scratch in a static device array.  Here it is
called through the C ABI on particle columns owned by the caller (torch
tensors) and must give the same result as st_DeviceLattice_track_until, the
entry point that allocates its scratch, on two calls in a row.  The file is
named to be collected last so that a run stopping at the first failure has
already run every other test.
"""

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _lib():
    from sixtracklib_gb300 import _native

    lib = _native.load()
    fn = lib.st_DeviceLattice_track_until_noalloc
    fn.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_int64, C.c_void_p]
    fn.restype = C.c_int32
    return lib, fn


def test_noalloc_matches_allocating_entry_point():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("GPU tests need a CUDA device")
    from sixtracklib_gb300 import _native, lattices
    from sixtracklib_gb300.device import DeviceTracker

    lib, noalloc = _lib()
    ring = lattices.synthetic_ring()  # streams through shared memory
    trk = DeviceTracker(ring.cbuffer, config="mode=fast")
    parts = lattices.polar_grid_particles(50_000, seed=77)
    base = torch.from_numpy(parts.block.copy().view(np.int64)).cuda()
    ref = base.clone()
    got = base.clone()
    stream = torch.cuda.current_stream().cuda_stream
    for until in (2, 4):  # two calls in a row
        st_ref = trk.track_until(ref, until)
        st_got = noalloc(trk._ptr, got.data_ptr(), got.shape[1], until, stream)
        assert st_got == st_ref == 0, _native.last_error()
        torch.cuda.synchronize()
        # same kernels, same arithmetic: identical columns
        assert torch.equal(got, ref)
    lost = int((ref[20] == 0).sum())
    assert 0 < lost < ref.shape[1]


def test_noalloc_allocates_no_device_memory():
    """After warm-up (the first call on the device and the allocating path),
    a call with more particles than any earlier allocating call leaves the
    device's free memory and torch's reserved memory unchanged: the
    allocating entry point would have had to grow its selection scratch."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("GPU tests need a CUDA device")
    from sixtracklib_gb300 import _native, lattices
    from sixtracklib_gb300.device import DeviceTracker

    lib, noalloc = _lib()
    trk = DeviceTracker(lattices.fodo_ring().cbuffer, config="mode=fast")
    stream = torch.cuda.current_stream().cuda_stream
    small = torch.from_numpy(lattices.gaussian_particles(1000, seed=3).block.copy()
                             .view(np.int64)).cuda()
    assert trk.track_until(small.clone(), 1) == 0
    assert noalloc(trk._ptr, small.data_ptr(), small.shape[1], 1, stream) == 0
    big = torch.from_numpy(lattices.gaussian_particles(900_000, seed=4).block.copy()
                           .view(np.int64)).cuda()
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    reserved0 = torch.cuda.memory_reserved()
    assert noalloc(trk._ptr, big.data_ptr(), big.shape[1], 2, stream) == 0, _native.last_error()
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    assert torch.cuda.memory_reserved() == reserved0
    assert int((big[19] == 2).sum()) > 0  # the call did track


def test_noalloc_rejects_oversized_calls():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("GPU tests need a CUDA device")
    from sixtracklib_gb300 import _native, lattices
    from sixtracklib_gb300.device import DeviceTracker

    lib, noalloc = _lib()
    trk = DeviceTracker(lattices.fodo_ring().cbuffer, config="mode=exact")
    cols = torch.zeros((21, 4), dtype=torch.int64, device="cuda")
    # the size check comes before any launch: nothing touches `cols`
    st = noalloc(trk._ptr, cols.data_ptr(), (1 << 20) + 1, 1,
                 torch.cuda.current_stream().cuda_stream)
    assert st == -1
    assert "1048576" in _native.last_error()
    assert int(cols.abs().sum()) == 0
