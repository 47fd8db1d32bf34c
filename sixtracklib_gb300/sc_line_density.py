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
from .beam_elements import Elements


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
