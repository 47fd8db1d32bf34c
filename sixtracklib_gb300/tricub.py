"""TriCub elements (python/sixtracklib/tricub.py).  The TriCub map is
disabled in the reference's default build (Settings.cmake.default) and in
this engine's default configuration: a lattice with a TriCub fails to
track.  The configuration key ``track_tricub`` ("enabled", "skip",
"disabled") selects the map per job or tracker, as SIXTRACKL_TRACK_TRICUB
selects it per reference build.  The TriCubData's table is gathered to the
GPU when the lattice is compiled; a job assigns its address to the TriCub
from a stored buffer (below), or the TriCub names TriCubData of its own
buffer."""

from __future__ import annotations

from .beam_elements import TriCub, TriCubData  # noqa: F401
from .buffer import ARCH_BEAM_ELEMENTS_BUFFER_ID, ARCH_ILLEGAL_BUFFER_ID


def TriCub_buffer_create_assign_address_item(track_job, be_tricub_index, tricub_data_buffer_id,
                                             tricub_data_index):
    """Add the assignment of TriCubData ``tricub_data_index`` of stored
    buffer ``tricub_data_buffer_id`` to the data_addr of TriCub
    ``be_tricub_index`` of the job's beam elements (tricub.py:71-105); True
    if a new item was added."""
    assert tricub_data_buffer_id != ARCH_ILLEGAL_BUFFER_ID
    assert (track_job.min_stored_buffer_id <= tricub_data_buffer_id
            <= track_job.max_stored_buffer_id)
    assert track_job.stored_buffer(tricub_data_buffer_id).num_objects > tricub_data_index
    before = track_job.num_assign_items(ARCH_BEAM_ELEMENTS_BUFFER_ID, tricub_data_buffer_id)
    track_job.add_assign_address_item(
        dest_elem_type_id=TriCub._typeid, dest_buffer_id=ARCH_BEAM_ELEMENTS_BUFFER_ID,
        dest_elem_index=be_tricub_index, dest_pointer_offset=TriCub.data_addr_offset(),
        src_elem_type_id=TriCubData._typeid, src_buffer_id=tricub_data_buffer_id,
        src_elem_index=tricub_data_index, src_pointer_offset=TriCubData.ptr_offset())
    return before < track_job.num_assign_items(ARCH_BEAM_ELEMENTS_BUFFER_ID,
                                               tricub_data_buffer_id)
