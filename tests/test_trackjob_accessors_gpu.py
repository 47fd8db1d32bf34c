"""The TrackJob and TrackJobNew / CudaTrackJob accessors of the C ABI
(common/track_job.h:139-400, common/track/track_job_base.h:53-189): particle
sets, buffers, output layout (elem-by-elem store first, then one block per
beam monitor), collect flags, push / collect, reset and clear, particle
addresses, on a job with two particle sets and two beam monitors."""

import ctypes as C

import numpy as np
import pytest

from sixtracklib_gb300 import ParticlesSet, _native, lattices
from sixtracklib_gb300.beam_elements import Elements

pytestmark = pytest.mark.gpu

VP, U64, U16, B, I64, U32, I32 = (C.c_void_p, C.c_uint64, C.c_uint16, C.c_bool, C.c_int64,
                                  C.c_uint32, C.c_int32)


@pytest.fixture(scope="module")
def L():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("GPU tests need a CUDA device")
    _native.load()
    L = C.CDLL(_native.lib_path())  # own prototypes, not the shared handle's
    sigs = [
        ("st_Buffer_new_on_data", [VP, U64], VP), ("st_Buffer_delete", [VP], None),
        ("st_Buffer_get_num_of_objects", [VP], U64),
        ("st_TrackJob_new_detailed", [C.c_char_p, VP, U64, VP, VP, VP, U64, C.c_char_p], VP),
        ("st_TrackJob_delete", [VP], None), ("st_TrackJob_clear", [VP], None),
        ("st_TrackJob_reset", [VP, VP, VP, VP], B),
        ("st_TrackJob_reset_with_output", [VP, VP, VP, VP, U64], B),
        ("st_TrackJob_reset_detailed", [VP, VP, U64, VP, VP, VP, U64], B),
        ("st_TrackJob_track_until", [VP, U64], I32),
        ("st_TrackJob_push", [VP, U16], None), ("st_TrackJob_collect_detailed", [VP, U16], None),
        ("st_TrackJob_collect_beam_elements", [VP], None),
        ("st_TrackJob_get_num_particle_sets", [VP], U64),
        ("st_TrackJob_get_particle_set_indices_begin", [VP], VP),
        ("st_TrackJob_get_particle_set_indices_end", [VP], VP),
        ("st_TrackJob_get_particle_set_index", [VP, U64], U64),
        ("st_TrackJob_get_total_num_particles_in_sets", [VP], U64),
        ("st_TrackJob_get_max_initial_turn_id", [VP], I64),
        ("st_TrackJob_get_particles_buffer", [VP], VP),
        ("st_TrackJob_get_const_particles_buffer", [VP], VP),
        ("st_TrackJob_get_beam_elements_buffer", [VP], VP),
        ("st_TrackJob_get_const_beam_elements_buffer", [VP], VP),
        ("st_TrackJob_get_const_output_buffer", [VP], VP),
        ("st_TrackJob_get_output_buffer", [VP], VP),
        ("st_TrackJob_has_output_buffer", [VP], B), ("st_TrackJob_owns_output_buffer", [VP], B),
        ("st_TrackJob_get_num_elem_by_elem_turns", [VP], U64),
        ("st_TrackJob_has_elem_by_elem_config", [VP], B),
        ("st_TrackJob_get_elem_by_elem_config_order", [VP], I64),
        ("st_TrackJob_is_elem_by_elem_config_rolling", [VP], B),
        ("st_TrackJob_get_default_elem_by_elem_config_rolling_flag", [VP], B),
        ("st_TrackJob_set_default_elem_by_elem_config_rolling_flag", [VP, B], None),
        ("st_TrackJob_has_beam_monitors", [VP], B),
        ("st_TrackJob_get_beam_monitor_indices_begin", [VP], VP),
        ("st_TrackJob_get_beam_monitor_indices_end", [VP], VP),
        ("st_TrackJob_get_beam_monitor_index", [VP, U64], U64),
        ("st_TrackJob_get_collect_flags", [VP], U16), ("st_TrackJob_set_collect_flags", [VP, U16], None),
        ("st_TrackJob_enable_collect_particles", [VP], None),
        ("st_TrackJob_disable_collect_particles", [VP], None),
        ("st_TrackJob_enable_collect_beam_elements", [VP], None),
        ("st_TrackJob_disable_collect_beam_elements", [VP], None),
        ("st_TrackJob_is_collecting_beam_elements", [VP], B),
        ("st_TrackJob_enable_collect_output", [VP], None),
        ("st_TrackJob_disable_collect_output", [VP], None),
        ("st_TrackJob_is_collecting_output", [VP], B),
        ("st_TrackJob_is_collecting_particles", [VP], B),
        ("st_TrackJob_requires_collecting", [VP], B),
        ("st_TrackJob_has_config_str", [VP], B), ("st_TrackJob_get_config_str", [VP], C.c_char_p),
        ("st_TrackJob_has_device_id_str", [VP], B),
        ("st_TrackJob_get_device_id_str", [VP], C.c_char_p),
        ("st_TrackJobNew_new_detailed", [C.c_char_p, VP, U64, VP, VP, VP, U64, C.c_char_p], VP),
        ("st_TrackJobNew_delete", [VP], None), ("st_TrackJobNew_clear", [VP], None),
        ("st_TrackJobNew_get_arch_id", [VP], U32), ("st_TrackJobNew_has_arch_string", [VP], B),
        ("st_TrackJobNew_get_num_particle_sets", [VP], U64),
        ("st_TrackJobNew_has_config_str", [VP], B),
        ("st_TrackJobNew_get_config_str", [VP], C.c_char_p),
        ("st_TrackJobNew_get_particles_buffer", [VP], VP),
        ("st_TrackJobNew_get_const_particles_buffer", [VP], VP),
        ("st_TrackJobNew_get_beam_elements_buffer", [VP], VP),
        ("st_TrackJobNew_get_const_beam_elements_buffer", [VP], VP),
        ("st_TrackJobNew_get_output_buffer", [VP], VP),
        ("st_TrackJobNew_get_const_output_buffer", [VP], VP),
        ("st_TrackJobNew_has_elem_by_elem_output", [VP], B),
        ("st_TrackJobNew_has_beam_monitor_output", [VP], B),
        ("st_TrackJobNew_get_elem_by_elem_output_buffer_offset", [VP], U64),
        ("st_TrackJobNew_get_beam_monitor_output_buffer_offset", [VP], U64),
        ("st_TrackJobNew_get_collect_flags", [VP], U16),
        ("st_TrackJobNew_set_collect_flags", [VP, U16], None),
        ("st_TrackJobNew_enable_collect_particles", [VP], None),
        ("st_TrackJobNew_disable_collect_particles", [VP], None),
        ("st_TrackJobNew_is_collecting_particles", [VP], B),
        ("st_TrackJobNew_requires_collecting", [VP], B),
        ("st_TrackJobNew_push", [VP, U16], U16),
        ("st_TrackJobNew_push_particles", [VP], I32),
        ("st_TrackJobNew_push_beam_elements", [VP], I32),
        ("st_TrackJobNew_push_output", [VP], I32),
        ("st_TrackJobNew_collect", [VP], I32),
        ("st_TrackJobNew_collect_beam_elements", [VP], I32),
        ("st_TrackJobNew_collect_output", [VP], I32),
        ("st_TrackJobNew_track_until", [VP, U64], I32),
        ("st_TrackJobNew_reset_with_output", [VP, VP, VP, VP, U64], I32),
        ("st_TrackJobNew_reset_detailed", [VP, VP, U64, VP, VP, VP, U64], I32),
        ("st_TrackJobNew_can_fetch_particle_addresses", [VP], B),
        ("st_TrackJobNew_has_particle_addresses", [VP], B),
        ("st_TrackJobNew_fetch_particle_addresses", [VP], I32),
        ("st_TrackJobNew_get_particle_addresses", [VP, U64], VP),
        ("st_TrackJobNew_clear_particle_addresses", [VP, U64], I32),
        ("st_TrackJobNew_clear_all_particle_addresses", [VP], I32),
    ]
    for name, args, res in sigs:
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res
    return L


def _setup(L):
    """Two particle sets (ids 0-3 and 10-12) and a lattice with beam
    monitors at objects 2 and 4; C buffers over numpy images (kept alive by
    the returned tuple)."""
    ps = ParticlesSet()
    for n, first in ((4, 0), (3, 10)):
        p = ps.Particles(num_particles=n)
        blk = lattices.gaussian_particles(n, seed=first + 1).block.copy()
        blk[17] = np.arange(first, first + n, dtype=np.int64).view(np.uint64)
        p.set_block(blk)
    e = Elements()
    e.Drift(length=1.0)
    e.Multipole(knl=[0.0, 0.01])
    e.BeamMonitor(num_stores=2, start=0, skip=1)
    e.Drift(length=1.0)
    e.BeamMonitor(num_stores=1, start=5, skip=1)
    pimg, eimg = ps.cbuffer.to_image(), e.cbuffer.to_image()
    pb = L.st_Buffer_new_on_data(pimg.ctypes.data, pimg.nbytes)
    eb = L.st_Buffer_new_on_data(eimg.ctypes.data, eimg.nbytes)
    assert pb and eb, _native.last_error()
    return pb, eb, pimg, eimg


def _column(L, pb, index, col):
    """Column `col` of the Particles object `index` of a C buffer (int64)."""
    L.st_Particles_buffer_get_particles.argtypes = [VP, U64]
    L.st_Particles_buffer_get_particles.restype = VP
    sp = L.st_Particles_buffer_get_particles(pb, index)
    arr = C.cast(sp, C.POINTER(C.c_uint64))
    n = int(arr[0])
    return np.ctypeslib.as_array(C.cast(arr[1 + col], C.POINTER(C.c_int64)), shape=(n,)).copy()


def _u64s(begin, end):
    n = (end - begin) // 8
    return list(np.ctypeslib.as_array(C.cast(begin, C.POINTER(C.c_uint64)), shape=(n,)))


def test_trackjob_accessors(L):
    pb, eb, pimg, eimg = _setup(L)
    idx = (C.c_uint64 * 2)(0, 1)
    job = L.st_TrackJob_new_detailed(b"cuda", pb, 2, idx, eb, None, 3, b"mode=exact")
    assert job, _native.last_error()
    try:
        assert L.st_TrackJob_get_num_particle_sets(job) == 2
        assert _u64s(L.st_TrackJob_get_particle_set_indices_begin(job),
                     L.st_TrackJob_get_particle_set_indices_end(job)) == [0, 1]
        assert L.st_TrackJob_get_particle_set_index(job, 1) == 1
        assert L.st_TrackJob_get_particle_set_index(job, 2) == 2 ** 64 - 1
        assert L.st_TrackJob_get_total_num_particles_in_sets(job) == 7
        assert L.st_TrackJob_get_max_initial_turn_id(job) == 0
        assert L.st_TrackJob_get_particles_buffer(job) == pb
        assert L.st_TrackJob_get_const_particles_buffer(job) == pb
        assert L.st_TrackJob_get_beam_elements_buffer(job) == eb
        assert L.st_TrackJob_get_const_beam_elements_buffer(job) == eb
        # job-owned output: the elem-by-elem store, then the two monitors
        assert L.st_TrackJob_has_output_buffer(job) and L.st_TrackJob_owns_output_buffer(job)
        ob = L.st_TrackJob_get_output_buffer(job)
        assert ob and L.st_TrackJob_get_const_output_buffer(job) == ob
        assert L.st_Buffer_get_num_of_objects(ob) == 3
        assert L.st_TrackJob_get_num_elem_by_elem_turns(job) == 3
        assert L.st_TrackJob_has_elem_by_elem_config(job)
        assert L.st_TrackJob_get_elem_by_elem_config_order(job) == 0
        assert L.st_TrackJob_get_default_elem_by_elem_config_rolling_flag(job)
        assert L.st_TrackJob_is_elem_by_elem_config_rolling(job)
        L.st_TrackJob_set_default_elem_by_elem_config_rolling_flag(job, False)
        assert not L.st_TrackJob_get_default_elem_by_elem_config_rolling_flag(job)
        assert L.st_TrackJob_has_beam_monitors(job)
        assert _u64s(L.st_TrackJob_get_beam_monitor_indices_begin(job),
                     L.st_TrackJob_get_beam_monitor_indices_end(job)) == [2, 4]
        assert L.st_TrackJob_get_beam_monitor_index(job, 1) == 4
        # collect flags: particles | output by default (track/definitions.h)
        assert L.st_TrackJob_get_collect_flags(job) == 0x05
        L.st_TrackJob_enable_collect_beam_elements(job)
        assert L.st_TrackJob_is_collecting_beam_elements(job)
        L.st_TrackJob_disable_collect_beam_elements(job)
        L.st_TrackJob_disable_collect_output(job)
        assert not L.st_TrackJob_is_collecting_output(job)
        L.st_TrackJob_enable_collect_output(job)
        L.st_TrackJob_disable_collect_particles(job)
        assert not L.st_TrackJob_is_collecting_particles(job)
        L.st_TrackJob_enable_collect_particles(job)
        assert L.st_TrackJob_get_collect_flags(job) == 0x05
        L.st_TrackJob_set_collect_flags(job, 0x03)
        assert L.st_TrackJob_get_collect_flags(job) == 0x03
        assert L.st_TrackJob_requires_collecting(job)
        assert L.st_TrackJob_has_config_str(job)
        assert L.st_TrackJob_get_config_str(job) == b"mode=exact"
        assert L.st_TrackJob_has_device_id_str(job)
        assert L.st_TrackJob_get_device_id_str(job).startswith(b"0.")
        # push / track / collect by flags: the particles advance one turn
        assert list(_column(L, pb, 1, 19)) == [0, 0, 0]  # at_turn
        L.st_TrackJob_push(job, 0x01)
        assert L.st_TrackJob_track_until(job, 1) == 0
        L.st_TrackJob_collect_detailed(job, 0x01)
        L.st_TrackJob_collect_beam_elements(job)
        assert list(_column(L, pb, 1, 19)) == [1, 1, 1]
        # reset: one set, no elem-by-elem output (monitors still write)
        assert L.st_TrackJob_reset(job, pb, eb, None)
        assert L.st_TrackJob_get_num_particle_sets(job) == 1
        assert not L.st_TrackJob_has_elem_by_elem_config(job)
        assert L.st_TrackJob_reset_with_output(job, pb, eb, None, 2)
        assert L.st_TrackJob_has_elem_by_elem_config(job)
        assert L.st_TrackJob_get_num_elem_by_elem_turns(job) == 2
        one = (C.c_uint64 * 1)(1)
        assert L.st_TrackJob_reset_detailed(job, pb, 1, one, eb, None, 0)
        assert L.st_TrackJob_get_particle_set_index(job, 0) == 1
        assert L.st_TrackJob_get_total_num_particles_in_sets(job) == 3
        L.st_TrackJob_clear(job)
        assert not L.st_TrackJob_has_output_buffer(job)
        assert not L.st_TrackJob_has_beam_monitors(job)
    finally:
        L.st_TrackJob_delete(job)
        L.st_Buffer_delete(pb)
        L.st_Buffer_delete(eb)


def test_trackjobnew_accessors(L):
    pb, eb, pimg, eimg = _setup(L)
    idx = (C.c_uint64 * 2)(0, 1)
    job = L.st_TrackJobNew_new_detailed(b"cuda", pb, 2, idx, eb, None, 0, b"mode=fast")
    assert job, _native.last_error()
    try:
        assert L.st_TrackJobNew_get_arch_id(job) == 3  # SIXTRL_ARCHITECTURE_CUDA
        assert L.st_TrackJobNew_has_arch_string(job)
        assert L.st_TrackJobNew_get_num_particle_sets(job) == 2
        assert L.st_TrackJobNew_has_config_str(job)
        assert L.st_TrackJobNew_get_config_str(job) == b"mode=fast"
        assert L.st_TrackJobNew_get_particles_buffer(job) == pb
        assert L.st_TrackJobNew_get_const_particles_buffer(job) == pb
        assert L.st_TrackJobNew_get_beam_elements_buffer(job) == eb
        assert L.st_TrackJobNew_get_const_beam_elements_buffer(job) == eb
        ob = L.st_TrackJobNew_get_output_buffer(job)
        assert ob and L.st_TrackJobNew_get_const_output_buffer(job) == ob
        assert not L.st_TrackJobNew_has_elem_by_elem_output(job)
        assert L.st_TrackJobNew_has_beam_monitor_output(job)
        assert L.st_TrackJobNew_get_beam_monitor_output_buffer_offset(job) == 0
        assert L.st_TrackJobNew_get_collect_flags(job) == 0x05
        L.st_TrackJobNew_disable_collect_particles(job)
        assert not L.st_TrackJobNew_is_collecting_particles(job)
        L.st_TrackJobNew_enable_collect_particles(job)
        L.st_TrackJobNew_set_collect_flags(job, 0x01)
        assert L.st_TrackJobNew_get_collect_flags(job) == 0x01
        assert L.st_TrackJobNew_requires_collecting(job)
        assert L.st_TrackJobNew_push(job, 0x07) == 0x07
        assert L.st_TrackJobNew_push_particles(job) == 0
        assert L.st_TrackJobNew_push_beam_elements(job) == 0
        assert L.st_TrackJobNew_push_output(job) == 0
        assert L.st_TrackJobNew_track_until(job, 2) == 0
        assert L.st_TrackJobNew_collect(job) == 0
        assert L.st_TrackJobNew_collect_beam_elements(job) == 0
        assert L.st_TrackJobNew_collect_output(job) == 0
        # particle addresses of the device copies
        assert L.st_TrackJobNew_can_fetch_particle_addresses(job)
        assert not L.st_TrackJobNew_has_particle_addresses(job)
        assert L.st_TrackJobNew_fetch_particle_addresses(job) == 0
        assert L.st_TrackJobNew_has_particle_addresses(job)
        addr = L.st_TrackJobNew_get_particle_addresses(job, 1)
        assert addr and C.cast(addr, C.POINTER(C.c_int64))[0] == 3
        assert L.st_TrackJobNew_clear_particle_addresses(job, 1) == 0
        assert not L.st_TrackJobNew_get_particle_addresses(job, 1)
        assert L.st_TrackJobNew_get_particle_addresses(job, 0)
        assert L.st_TrackJobNew_clear_all_particle_addresses(job) == 0
        assert not L.st_TrackJobNew_has_particle_addresses(job)
        # reset with an elem-by-elem output (the particles are at turn 2
        # now: stores up to turn 5), then with one particle set
        assert L.st_TrackJobNew_reset_with_output(job, pb, eb, None, 5) == 0
        assert L.st_TrackJobNew_has_elem_by_elem_output(job)
        assert L.st_TrackJobNew_get_elem_by_elem_output_buffer_offset(job) == 0
        assert L.st_TrackJobNew_get_beam_monitor_output_buffer_offset(job) == 1
        one = (C.c_uint64 * 1)(1)
        assert L.st_TrackJobNew_reset_detailed(job, pb, 1, one, eb, None, 0) == 0
        assert L.st_TrackJobNew_get_num_particle_sets(job) == 1
        L.st_TrackJobNew_clear(job)
        assert not L.st_TrackJobNew_has_beam_monitor_output(job)
    finally:
        L.st_TrackJobNew_delete(job)
        L.st_Buffer_delete(pb)
        L.st_Buffer_delete(eb)
