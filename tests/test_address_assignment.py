"""Stored buffers and address assignment on the CPU (python/sixtracklib/
buffer.py, trackjob.py:1833-2290, sc_line_density.py:113-150): the C-side
buffer copies a TrackJob works on, the assignment of line-density tables
to interpolated space-charge kicks, and the in-place refresh that carries
later edits of a lattice to the engine.  The tracking checks use the C
oracle, which dereferences a kick's table address as the reference's CPU
tracking does."""

import numpy as np
import pytest

from sixtracklib_gb300 import lattices
from sixtracklib_gb300.beam_elements import (TYPE_LINE_DENSITY_PROF_DATA,
                                             TYPE_SC_INTERPOLATED_PROF, Elements,
                                             LineDensityProfileData, SCInterpolatedProfile)
from sixtracklib_gb300.buffer import (ARCH_BEAM_ELEMENTS_BUFFER_ID, AddressAssignments,
                                      AssignAddressItem, CBufferHandle)


def _tables():
    z = np.linspace(-0.3, 0.3, 41)
    prof = np.exp(-0.5 * (z / 0.1) ** 2) * 1e12
    t = Elements()
    t.LineDensityProfileData(values=prof, z0=-0.3, dz=float(z[1] - z[0]), method="linear",
                             capacity=48)
    t.LineDensityProfileData(values=prof * 1.1, z0=-0.3, dz=float(z[1] - z[0]), method="cubic")
    return t


def _ring_without_addresses(n_kicks=6):
    e = lattices.fodo_ring()
    first = len(e)
    for k in range(n_kicks):
        e.SCInterpolatedProfile(number_of_particles=1e11, length=0.5, sigma_x=1e-3,
                                sigma_y=1.2e-3 if k % 2 else 1e-3, interpol_data_addr=0,
                                line_density_prof_fallback=5e11, min_sigma_diff=1e-10)
    return e, first


def _item(sc_index, table_index, stored_id=1024):
    return AssignAddressItem(
        dest_elem_type_id=TYPE_SC_INTERPOLATED_PROF, dest_buffer_id=ARCH_BEAM_ELEMENTS_BUFFER_ID,
        dest_elem_index=sc_index,
        dest_pointer_offset=SCInterpolatedProfile.interpol_data_addr_offset(),
        src_elem_type_id=TYPE_LINE_DENSITY_PROF_DATA, src_buffer_id=stored_id,
        src_elem_index=table_index, src_pointer_offset=LineDensityProfileData.ptr_offset())


def test_assignment_tracks_like_table_addresses(oracle):
    """Kicks whose tables are assigned from a stored buffer track exactly
    like the same kicks given the tables' addresses directly."""
    from sixtracklib_gb300.sc_line_density import LineDensityBuffer

    tables = _tables()
    stored = CBufferHandle(tables.cbuffer)
    e, first = _ring_without_addresses()
    a = AddressAssignments()
    for k in range(6):
        a.add(_item(first + k, k % 2))
    a.add(_item(first, 0))  # the same item again: not added twice
    assert len(a.items) == 6 and a.index_of(_item(first + 3, 1)) == 3
    written = a.perform({1024: stored}, {ARCH_BEAM_ELEMENTS_BUFFER_ID: e.cbuffer})
    assert written == {ARCH_BEAM_ELEMENTS_BUFFER_ID}
    for k in range(6):
        assert e.get(first + k).interpol_data_addr == stored.object_info(k % 2)[0]
    # the same tables handed out as plain addresses
    direct = LineDensityBuffer()
    z = np.linspace(-0.3, 0.3, 41)
    prof = np.exp(-0.5 * (z / 0.1) ** 2) * 1e12
    i0 = direct.add(prof, z0=-0.3, dz=float(z[1] - z[0]), method="linear", capacity=48)
    i1 = direct.add(prof * 1.1, z0=-0.3, dz=float(z[1] - z[0]), method="cubic")
    e2, _ = _ring_without_addresses()
    for k in range(6):
        obj = e2.cbuffer.objects[first + k]
        obj.words[6] = np.uint64(direct.address(i0 if k % 2 == 0 else i1))
    e2.cbuffer.touch()
    p = lattices.gaussian_particles(256, seed=4, sz=0.12).block
    got, exp = p.copy(), p.copy()
    assert oracle.track_until(e.cbuffer.to_image(), got, 5) == 0
    assert oracle.track_until(e2.cbuffer.to_image(), exp, 5) == 0
    assert np.array_equal(got, exp)
    # and differently from the fallback density: the tables were used
    e3, _ = _ring_without_addresses()
    fb = p.copy()
    assert oracle.track_until(e3.cbuffer.to_image(), fb, 5) == 0
    assert not np.array_equal(got, fb)
    stored.free()


def test_assignment_checks():
    tables = _tables()
    stored = CBufferHandle(tables.cbuffer)
    e, first = _ring_without_addresses(2)
    dst = {ARCH_BEAM_ELEMENTS_BUFFER_ID: e.cbuffer}
    bad_type = _item(first, 0)
    bad_type.src_elem_type_id = 999
    bad_dest = _item(0, 0)  # element 0 is a drift
    bad_index = _item(first, 7)
    for it in (bad_type, bad_dest, bad_index):
        a = AddressAssignments()
        a.add(it)
        with pytest.raises((RuntimeError, IndexError)):
            a.perform({1024: stored}, dst)
    a = AddressAssignments()
    a.add(_item(first, 0, stored_id=2048))
    with pytest.raises(RuntimeError, match="unknown buffers"):
        a.perform({1024: stored}, dst)
    with pytest.raises(ValueError):
        AddressAssignments.make(dest_buffer_id=2, src_buffer_id=1024)
    stored.free()


def test_refresh_carries_edits_to_the_copy(oracle):
    """A TrackJob's C-side lattice copy follows edits made after it was
    created (set_knl, assigned addresses); a changed structure is refused."""
    e = lattices.fodo_ring()
    h = CBufferHandle(e.cbuffer)
    e.get(1).set_knl(0.055, 1)
    h.refresh(e.cbuffer)
    img = h.image()
    p = lattices.gaussian_particles(64, seed=2).block
    a, b = p.copy(), p.copy()
    assert oracle.track_until(img, a, 3) == 0
    assert oracle.track_until(e.cbuffer.to_image(), b, 3) == 0
    assert np.array_equal(a, b)
    e.Drift(length=1.0)
    with pytest.raises(RuntimeError, match="reset"):
        h.refresh(e.cbuffer)
    h.free()


def test_trackjob_host_logic_without_engine(oracle):
    """The TrackJob's stored-buffer and assignment methods, on a job
    assembled without its engine part (no GPU here; the engine's push of a
    null job is a no-op): ids, item bookkeeping, commit checks, and the
    C-side lattice copy carrying the assigned addresses."""
    from sixtracklib_gb300.buffer import AddressAssignments
    from sixtracklib_gb300.particles import ParticlesSet
    from sixtracklib_gb300.sc_line_density import LineDensityProfileData_create_buffer_assignment
    from sixtracklib_gb300.trackjob import TrackJob

    tables = _tables()
    e, first = _ring_without_addresses(4)
    ps = ParticlesSet()
    ps.Particles(num_particles=8)
    job = TrackJob.__new__(TrackJob)
    job._lib = __import__("sixtracklib_gb300._native", fromlist=["load"]).load()
    job.ptr_st_track_job = None
    job._stored, job._next_stored_id = {}, 1024
    job._assign, job._assigned, job._last_status = AddressAssignments(), False, 0
    job._particles_buffer, job._beam_elements_buffer = ps.cbuffer, e.cbuffer
    job._c_particles, job._c_elements = CBufferHandle(ps.cbuffer), CBufferHandle(e.cbuffer)
    job._c_output = None

    assert job.min_stored_buffer_id == 0 and not job.has_stored_buffers
    bid = job.add_stored_buffer(cbuffer=tables)
    assert bid == 1024 and job.add_stored_buffer(size=64) == 1025
    assert (job.min_stored_buffer_id, job.max_stored_buffer_id) == (1024, 1025)
    assert job.owns_stored_buffer(1025) and not job.owns_stored_buffer(1024)
    assert job.remove_stored_buffer(1025) == 0 and job.num_stored_buffers == 1
    assert job.add_stored_buffer() == 0
    for k in range(4):
        assert LineDensityProfileData_create_buffer_assignment(job, first + k, bid, k % 2)
    assert job.total_num_assign_items == 4 and job.has_assign_items(2, bid)
    assert job.has_assign_item(dest_buffer_id=2, src_buffer_id=bid, index=3)
    item = job.ptr_assign_address_item(dest_buffer_id=2, src_buffer_id=bid, index=2)
    assert job.index_of_assign_address_item(item) == 2
    job.commit_address_assignments()
    job.assign_all_addresses()
    got, exp = (lattices.gaussian_particles(128, seed=9, sz=0.12).block.copy() for _ in range(2))
    assert oracle.track_until(job._c_elements.image(), got, 4) == 0  # the engine's copy
    assert oracle.track_until(e.cbuffer.to_image(), exp, 4) == 0
    assert np.array_equal(got, exp)
    assert e.get(first + 1).interpol_data_addr == job._stored[bid][1].object_info(1)[0]
    job.add_assign_address_item(dest_elem_type_id=TYPE_SC_INTERPOLATED_PROF, dest_buffer_id=2,
                                dest_elem_index=first, dest_pointer_offset=48,
                                src_elem_type_id=TYPE_LINE_DENSITY_PROF_DATA,
                                src_buffer_id=bid, src_elem_index=5, src_pointer_offset=0)
    with pytest.raises(RuntimeError):
        job.commit_address_assignments()
    with pytest.raises(ValueError):
        job.add_assign_address_item(dest_buffer_id=2)
    for h in (job._c_particles, job._c_elements):
        h.free()


def test_pull_into_brings_back_c_side_writes():
    """What the engine writes into its lattice copy (a monitor's particle-id
    range at job set-up) comes back into the Python lattice; pointer fields
    keep their Python form, so the lattice still serialises the same way."""
    import ctypes as C

    from sixtracklib_gb300.buffer import CBufferHandle

    e = lattices.fodo_ring()
    bm = len(e)
    e.BeamMonitor(num_stores=4, start=0, skip=1)
    h = CBufferHandle(e.cbuffer)
    b, t, s = h.object_info(bm)
    w = C.cast(C.c_void_p(b), C.POINTER(C.c_uint64))
    w[4], w[5] = 99, 3  # max / min particle id
    img0 = e.cbuffer.to_image().copy()
    h.pull_into(e.cbuffer)
    m = e.get(bm)
    assert (m.max_particle_id, m.min_particle_id) == (99, 3)
    diff = np.nonzero(e.cbuffer.to_image() != img0)[0]
    assert diff.size == 2  # only the two id fields changed
    np.testing.assert_array_equal(e.get(1).bal, lattices.fodo_ring().get(1).bal)
    h.free()


def test_buffer_class(tmp_path):
    """The C-side buffer wrapper (buffer.py:92-430): construction from a
    Python buffer, a size, capacities, a file and raw data; capacities,
    reserve / reset / clear; file round trips, with normalized addresses
    giving the Python writer's bytes."""
    import ctypes as Ct

    from sixtracklib_gb300 import lattices
    from sixtracklib_gb300.buffer import Buffer
    from sixtracklib_gb300.cbuffer import CBuffer

    e = lattices.fodo_ring()
    b = Buffer.from_cbuffer(e)
    assert b.maps_to_cbuffer and not b.owns_buffer and b.owns_pointer
    assert b.num_objects == len(e) and b.slot_size == 8 and b.header_size == 64
    assert b.data_end_addr - b.data_begin_addr == b.size <= b.capacity
    assert not b.needs_remapping and b.remap() is b and b.last_status_success
    assert b.num_garbage_ranges == 0 and b.max_num_objects >= b.num_objects
    e.get(0).length = 3.25  # a Python-side edit reaches the copy on refresh
    b.refresh()
    assert np.array_equal(CBuffer.from_image(b.image()).objects[0].words,
                          e.cbuffer.objects[0].words)
    path = str(tmp_path / "lattice.bin")
    b.write_to_file(path, normalized_base_addr=4096)
    raw = np.fromfile(path, dtype=np.uint64)
    assert raw[0] == 4096 and all(4096 <= raw[k] < 4096 + raw[1] for k in (3, 4, 5, 6))
    back = CBuffer.fromfile(path)
    assert [o.typeid for o in back.objects] == [o.typeid for o in e.cbuffer.objects]
    assert all(np.array_equal(x.words, y.words) for x, y in zip(back.objects, e.cbuffer.objects))
    f = Buffer(path_to_file=path)
    assert f.num_objects == len(e) and f.owns_buffer and f.is_owner
    g = Buffer(size=0).read_from_file(path)
    assert g.num_objects == len(e)
    img = e.cbuffer.to_image()
    r = Buffer(ptr_data=Ct.c_void_p(img.ctypes.data))
    assert r.num_objects == len(e)
    d = Buffer(num_objects=10, num_slots=100, num_dataptrs=5)
    assert (d.max_num_objects, d.max_num_slots, d.max_num_dataptrs) == (10, 100, 5)
    d.reserve(20, 200, 8, 0)
    assert (d.max_num_objects, d.max_num_slots, d.max_num_dataptrs) == (20, 200, 8)
    cap = d.capacity
    d.reserve_capacity(cap + 4096)
    assert d.capacity >= cap + 4096
    f.clear()
    assert f.num_objects == 0
    g.reset(max_num_objects=4)
    assert g.num_objects == 0 and g.max_num_objects == 4
    with pytest.raises(RuntimeError):
        g.write_to_file("")
