"""Line-density tables for the interpolated space-charge kick.

The reference keeps ``NS(LineDensityProfileData)`` objects in a buffer of
their own and writes the address of one into each
``NS(SCInterpolatedProfile)`` (its ``interpol_data_addr`` field, a plain
address that the CPU tracking dereferences; python/sixtracklib/
sc_line_density.py).  :class:`LineDensityBuffer` is that separate buffer: it
holds the tables in engine-owned host memory (an ``st_Buffer``) and hands
out their addresses.  The engine copies a table into the compiled lattice
when the lattice is compiled, so the buffer must stay alive until then (and
while the C oracle or the reference track the lattice).
"""

from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native
from .beam_elements import Elements, LineDensityProfileData  # noqa: F401  (sc_line_density.py)


class LineDensityBuffer:
    def __init__(self):
        self.elements = Elements()
        self._buf = None
        self._lib = None

    def add(self, values, z0: float, dz: float, method="linear", capacity=None) -> int:
        """Append a table (derivatives prepared as the reference does);
        returns its index.  Adding invalidates earlier addresses."""
        if self._buf is not None:
            self._release()
        self.elements.LineDensityProfileData(values=values, z0=z0, dz=dz, method=method,
                                             capacity=capacity)
        return len(self.elements) - 1

    def address(self, index: int) -> int:
        """Host address of table `index` (for ``interpol_data_addr``)."""
        if self._buf is None:
            self._lib = _native.load()
            img = np.ascontiguousarray(self.elements.cbuffer.to_image(), dtype=np.uint64)
            self._buf = self._lib.st_Buffer_new_on_data(img.ctypes.data, img.nbytes)
            if not self._buf:
                raise RuntimeError("st_Buffer_new_on_data: " + _native.last_error())
        obj = self._lib.st_Buffer_get_const_object(self._buf, int(index))
        if not obj:
            raise IndexError(index)
        return int(C.cast(obj, C.POINTER(C.c_uint64))[0])

    def _release(self):
        if self._buf is not None and self._lib is not None:
            self._lib.st_Buffer_delete(self._buf)
        self._buf = None

    def __del__(self):
        try:
            self._release()
        except Exception:
            pass


def LineDensityProfileData_create_buffer_assignment(track_job, be_sc_index, interpol_buffer_id,
                                                    lp_data_index):
    """Add the assignment of LineDensityProfileData ``lp_data_index`` of the
    job's stored buffer ``interpol_buffer_id`` to the interpol_data_addr of
    SCInterpolatedProfile ``be_sc_index`` of the job's beam elements
    (sc_line_density.py:113-150); True if a new item was added.  The
    addresses are written by ``track_job.assign_all_addresses()``."""
    from .beam_elements import (TYPE_LINE_DENSITY_PROF_DATA, TYPE_SC_INTERPOLATED_PROF,
                                LineDensityProfileData, SCInterpolatedProfile)
    from .buffer import ARCH_BEAM_ELEMENTS_BUFFER_ID, ARCH_ILLEGAL_BUFFER_ID

    assert interpol_buffer_id != ARCH_ILLEGAL_BUFFER_ID
    assert track_job.min_stored_buffer_id <= interpol_buffer_id <= track_job.max_stored_buffer_id
    assert track_job.stored_buffer(interpol_buffer_id).num_objects > lp_data_index
    before = track_job.num_assign_items(ARCH_BEAM_ELEMENTS_BUFFER_ID, interpol_buffer_id)
    track_job.add_assign_address_item(
        dest_elem_type_id=TYPE_SC_INTERPOLATED_PROF, dest_buffer_id=ARCH_BEAM_ELEMENTS_BUFFER_ID,
        dest_elem_index=be_sc_index,
        dest_pointer_offset=SCInterpolatedProfile.interpol_data_addr_offset(),
        src_elem_type_id=TYPE_LINE_DENSITY_PROF_DATA, src_buffer_id=interpol_buffer_id,
        src_elem_index=lp_data_index, src_pointer_offset=LineDensityProfileData.ptr_offset())
    return before < track_job.num_assign_items(ARCH_BEAM_ELEMENTS_BUFFER_ID, interpol_buffer_id)
