"""The stcommon CBuffer helpers (st_Buffer_new_mapped_on_cbuffer,
st_Particles_cbuffer_get_particles, st_OutputBuffer_create_output_cbuffer)
and string helpers, along the flows of the reference's
tests/python/test_output_buffer.py and test_cbuffer_st_buffer.py, on the
CPU."""

import ctypes as C

import numpy as np

from sixtracklib_gb300 import Elements, ParticlesSet
from sixtracklib_gb300 import stcommon as st


def _ring_with_monitors():
    e = Elements()
    e.Drift(length=1.0)
    e.BeamMonitor(num_stores=3, start=0, skip=1)
    e.Drift(length=2.0)
    e.BeamMonitor(num_stores=2, start=5, skip=2)
    e.Cavity(voltage=1e6, frequency=4e8, lag=180.0)
    return e


def _particles(n=5, turn=0):
    ps = ParticlesSet()
    ps.Particles(num_particles=n, particle_id=np.arange(n), at_turn=turn)
    return ps


def test_output_buffer_flow():
    """calculate params -> mapped output buffer -> prepare, as the
    reference's test_output_buffer.py does it, then the one-call helper."""
    e, ps = _ring_with_monitors(), _particles()
    pb = st.st_Buffer_new_mapped_on_cbuffer(ps.cbuffer)
    eb = st.st_Buffer_new_mapped_on_cbuffer(e.cbuffer)
    p = st.st_Particles_buffer_get_particles(pb, 0)
    assert p and st.st_Particles_get_num_of_particles(p) == 5
    sizes = [C.c_uint64(0) for _ in range(4)]
    assert st.st_OutputBuffer_calculate_output_buffer_params(
        eb, p, 10, *[C.byref(x) for x in sizes], st.st_Buffer_get_slot_size(pb)) == 0
    n_obj, n_slots, n_ptrs, n_garbage = (x.value for x in sizes)
    # 10 turns x 5 elements x 5 ids elem by elem, 3 and 2 stores x 5 ids
    assert (n_obj, n_ptrs, n_garbage) == (3, 63, 0)
    assert n_slots == 3 * 22 + 21 * (250 + 15 + 10)
    out = st.st_Buffer_new_detailed(n_obj, n_slots, n_ptrs, n_garbage, 0)
    ebe, mon, turn = C.c_uint64(9), C.c_uint64(9), C.c_int64(-1)
    assert st.st_OutputBuffer_prepare(eb, out, p, 10, C.byref(ebe), C.byref(mon),
                                      C.byref(turn)) == 0
    assert (ebe.value, mon.value, turn.value) == (0, 1, 0)
    assert st.st_Buffer_get_num_of_objects(out) == n_obj
    for b in (pb, eb, out):
        st.st_Buffer_delete(b)

    cb, ebe_off, mon_off, min_turn = st.st_OutputBuffer_create_output_cbuffer(
        e, ps, until_turn_elem_by_elem=10)
    assert (cb.n_objects, ebe_off, mon_off, min_turn) == (3, 0, 1, 0)
    assert [o.ints()[0] for o in cb.objects] == [250, 15, 10]
    # the monitors' particle-id ranges were written back into the lattice
    mons = [e.get(i) for i in (1, 3)]
    assert [(m.min_particle_id, m.max_particle_id) for m in mons] == [(0, 4), (0, 4)]


def test_output_cbuffer_without_outputs():
    e = Elements()
    e.Drift(length=1.0)
    assert st.st_OutputBuffer_create_output_cbuffer(e, _particles()) == (None, -1, -1, -1)


def test_output_cbuffer_starts_at_the_first_turn():
    """Particles already at turn 3: the monitor that started at turn 0 gets
    no block, the one starting at turn 5 does; elem-by-elem covers turns
    3..5 of 5 elements."""
    cb, ebe_off, mon_off, min_turn = st.st_OutputBuffer_create_output_cbuffer(
        _ring_with_monitors(), _particles(4, turn=3), until_turn_elem_by_elem=6)
    assert (ebe_off, mon_off, min_turn) == (0, 1, 3)
    assert [o.ints()[0] for o in cb.objects] == [4 * 5 * 3, 4 * 2]


def test_cbuffer_particles_pointer_and_difference():
    """test_cbuffer_st_buffer.py: the particles of a CBuffer seen through the
    C ABI equal those of a C buffer made from the same data, and their
    difference is zero."""
    ps = _particles(6)
    ps.particles[0].x[:] = np.linspace(-1e-3, 1e-3, 6)
    pb = st.st_Buffer_new_mapped_on_cbuffer(ps.cbuffer)
    assert st.st_Particles_buffer_get_num_of_particle_blocks(pb) == 1
    assert st.st_Particles_buffer_get_total_num_of_particles(pb) == 6
    p = st.st_Particles_buffer_get_particles(pb, 0)
    q = st.st_Particles_cbuffer_get_particles(ps.cbuffer, 0)
    assert q and q != p and st.st_Particles_get_num_of_particles(q) == 6
    diff_buf = st.st_Buffer_new(0)
    diff = st.st_Particles_new(diff_buf, 6)
    st.st_Particles_calculate_difference(p, q, diff)
    cols = C.cast(diff, C.POINTER(C.c_uint64))
    for c in range(1, 22):  # every column of the difference is zero
        col = C.cast(C.c_void_p(cols[c]), C.POINTER(C.c_uint64))
        assert all(col[k] == 0 for k in range(6))
    assert st.st_Particles_cbuffer_get_particles(_ring_with_monitors(), 0) is None
    for b in (pb, diff_buf):
        st.st_Buffer_delete(b)


def test_string_helpers_and_id_pair():
    s = st.string_to_encoded_ctypes_str(" cuda ")
    assert s.value == b"cuda"
    assert st.ctypes_str_to_decoded_string(s) == "cuda"
    assert st.ctypes_str_to_decoded_string(b"0.0\0junk") == "0.0"
    assert st.string_to_encoded_ctypes_str(None) is None
    pair = st.st_TrackJobDestSrcBufferIds(3, 1024)
    assert (pair.dest_buffer_id, pair.src_buffer_id) == (3, 1024)
    assert C.sizeof(pair) == 16 and not st.st_NullTrackJobDestSrcBufferIds
