"""C-side buffers of a TrackJob and address assignment
(python/sixtracklib/buffer.py:69-90, trackjob.py:1943-2035,
common/buffer/assign_address_item.h).

A TrackJob works on C-side ``st_Buffer`` copies of the caller's Python
buffers (:class:`CBufferHandle`); ``refresh`` writes the Python buffer's
current contents into that copy object by object, with pointer fields and
links relocated to the copy's addresses, so edits made after the job was
created (strengths, assigned addresses) reach the engine on the next push.

Address assignment: an :class:`AssignAddressItem` names a pointer field of
one object (destination: buffer id, object index, type id, byte offset in
the object) and a source (buffer id, object index, type id, byte offset);
performing it writes ``begin address of the source object + source
offset`` into the destination field, after the reference's checks (type
ids match, the offsets lie inside the objects, 8-byte alignment).  The
engine dereferences such an address when it compiles the lattice (for
example an SCInterpolatedProfile's ``interpol_data_addr``, copying the
LineDensityProfileData it points at), so the source buffer must stay
alive: a TrackJob keeps its stored buffers.
"""

from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native
from .beam_elements import _Element
from .cbuffer import CBuffer

# common/control/definitions.h:134-168
ARCH_ILLEGAL_BUFFER_ID = 0
ARCH_PARTICLES_BUFFER_ID = 1
ARCH_BEAM_ELEMENTS_BUFFER_ID = 2
ARCH_OUTPUT_BUFFER_ID = 3
ARCH_ELEM_BY_ELEM_CONFIG_BUFFER_ID = 4
ARCH_PARTICLE_ADDR_BUFFER_ID = 5
ARCH_MIN_USER_DEFINED_BUFFER_ID = 1024
ARCH_EXTERNAL_BUFFER_ID = 1024
ARCH_MAX_USER_DEFINED_BUFFER_ID = 0xFFFFFFFFFFFFFFFE

TYPE_ASSIGN_ADDRESS_ITEM = 513


def get_cbuffer_from_obj(obj):
    """The CBuffer of a buffer or of an object holding one, else None
    (buffer.py:81-89)."""
    if obj is None:
        return None
    if isinstance(obj, CBuffer):
        return obj
    for attr in ("cbuffer", "_cbuffer"):
        cb = getattr(obj, attr, None)
        if isinstance(cb, CBuffer):
            return cb
    return None


class CBufferHandle:
    """A C-side st_Buffer holding a copy of a Python CBuffer image."""

    def __init__(self, cbuffer: CBuffer):
        self._lib = _native.load()
        img = cbuffer.to_image()
        self.ptr = self._lib.st_Buffer_new_on_data(img.ctypes.data, img.nbytes)
        if not self.ptr:
            raise RuntimeError("st_Buffer_new_on_data failed: " + _native.last_error())

    def object_info(self, index: int):
        """(begin address, type id, size in bytes) of object ``index``."""
        n = self._lib.st_Buffer_get_num_of_objects(self.ptr)
        if not 0 <= index < n:
            raise IndexError(f"object {index} outside a buffer of {n} objects")
        o = C.cast(self._lib.st_Buffer_get_const_object(self.ptr, int(index)),
                   C.POINTER(C.c_uint64))
        return int(o[0]), int(o[1]), int(o[2])

    def image(self) -> np.ndarray:
        n = self._lib.st_Buffer_get_size(self.ptr)
        data = self._lib.st_Buffer_get_const_data_begin(self.ptr)
        return np.ctypeslib.as_array(C.cast(data, C.POINTER(C.c_uint64)), shape=(n // 8,)).copy()

    def refresh(self, cbuffer: CBuffer) -> None:
        """Write the Python buffer's objects into this copy in place.  The
        structure must be the one the copy was made from (same objects,
        types and sizes); a changed structure needs a new copy (reset)."""
        n = self._lib.st_Buffer_get_num_of_objects(self.ptr)
        if n != len(cbuffer.objects):
            raise RuntimeError(f"buffer structure changed ({len(cbuffer.objects)} objects, "
                               f"the job's copy has {n}): reset the job")
        begins = [self.object_info(i) for i in range(n)]
        for i, obj in enumerate(cbuffer.objects):
            b, t, s = begins[i]
            if t != obj.typeid or s != obj.words.nbytes:
                raise RuntimeError(f"object {i} changed type or size: reset the job")
            w = obj.words.copy()
            for f in obj.ptr_fields:
                w[f] = b + 8 * int(obj.words[f])
            for f, target in obj.links:
                w[f] = begins[target][0]
            C.memmove(b, w.ctypes.data, s)

    def pull_into(self, cbuffer: CBuffer) -> None:
        """Copy this copy's objects back into the Python buffer (the
        reference's buffers are one memory on both sides, so what its
        TrackJob writes -- a monitor's particle-id range at set-up -- is
        seen by the caller); pointer and link fields keep their Python
        form."""
        n = self._lib.st_Buffer_get_num_of_objects(self.ptr)
        if n != len(cbuffer.objects):
            raise RuntimeError("buffer structure changed: reset the job")
        for i, obj in enumerate(cbuffer.objects):
            b, t, s = self.object_info(i)
            if t != obj.typeid or s != obj.words.nbytes:
                raise RuntimeError(f"object {i} changed type or size: reset the job")
            cw = np.ctypeslib.as_array(C.cast(C.c_void_p(b), C.POINTER(C.c_uint64)),
                                       shape=(s // 8,))
            keep = sorted(set(obj.ptr_fields) | {f for f, _ in obj.links})
            saved = obj.words[keep].copy()
            obj.words[:] = cw
            obj.words[keep] = saved
        cbuffer.touch()

    def free(self):
        if self.ptr:
            self._lib.st_Buffer_delete(self.ptr)
            self.ptr = None


class Buffer:
    """A C-side NS(Buffer) (buffer.py:92-430).

    Made from a Python buffer (``cbuffer``: a C-side copy of its image, which
    ``refresh`` brings up to date after Python-side edits -- the reference
    maps the same memory instead), an existing ``st_Buffer`` pointer
    (``ptr_ext_buffer``, owned only if asked), a CObjects file, raw image
    data, or empty with a byte ``size`` or with object / slot / dataptr
    capacities.  A TrackJob's stored buffer is returned as a Buffer over the
    job's copy (owned by the job)."""

    maps_to_cbuffer = property(lambda self: self._cbuffer is not None and bool(self.pointer))

    def __init__(self, cbuffer=None, ptr_ext_buffer=None, owns_pointer=None, owns_buffer=None,
                 ptr_data=None, path_to_file=None, size=0, num_objects=None, num_slots=None,
                 num_dataptrs=None, num_garbage_ranges=None, buffer_flags=None, slot_size=8,
                 _handle=None):
        self._lib = _native.load()
        self._last_status = 0
        self._owns_buffer = self._owns_pointer = True
        self._cbuffer = get_cbuffer_from_obj(cbuffer)
        self._handle = _handle
        self._frees_handle = False
        self._ptr = None
        if _handle is not None:  # a TrackJob's copy: the job owns it
            self._owns_buffer = self._owns_pointer = False
        elif self._cbuffer is not None:
            # the Python buffer owns the data, as with the reference's mapping
            self._handle = CBufferHandle(self._cbuffer)
            self._frees_handle = True
            self._owns_buffer = False
        elif ptr_ext_buffer:
            self._ptr = ptr_ext_buffer
            self._owns_pointer = owns_pointer is True
            self._owns_buffer = owns_buffer is True
        elif path_to_file:
            self._ptr = self._lib.st_Buffer_new_from_file(str(path_to_file).encode())
        elif ptr_data:
            nbytes = C.cast(ptr_data, C.POINTER(C.c_uint64))[1]  # header word 1: the size
            self._ptr = self._lib.st_Buffer_new_on_data(ptr_data, int(nbytes))
        elif num_objects is not None and num_slots is not None and num_dataptrs is not None:
            self._ptr = self._lib.st_Buffer_new_detailed(
                int(num_objects), int(num_slots), int(num_dataptrs),
                int(num_garbage_ranges or 0), int(buffer_flags or 0))
        else:
            self._ptr = self._lib.st_Buffer_new(int(size or 0))
        if not self.pointer:
            raise RuntimeError("unable to create the buffer: " + _native.last_error())

    @classmethod
    def from_cbuffer(cls, obj, owns_buffer=False, owns_pointer=True, **kwargs):
        cb = get_cbuffer_from_obj(obj)
        if cb is None:
            raise ValueError(f"Unable to obtain cbuffer for {obj}")
        return cls(cbuffer=cb, owns_buffer=owns_buffer, owns_pointer=owns_pointer, **kwargs)

    def __del__(self):
        try:
            if self._frees_handle:
                self._handle.free()
                self._frees_handle = False
            elif self._ptr and self._owns_pointer:
                self._lib.st_Buffer_delete(self._ptr)
            self._ptr = None
        except Exception:
            pass

    # ------------------------------------------------------------ queries
    @property
    def pointer(self):
        return self._handle.ptr if self._handle is not None else self._ptr

    @property
    def cbuffer(self):
        return self._cbuffer

    @property
    def last_status(self):
        return self._last_status

    @property
    def last_status_success(self):
        return self._last_status == 0

    @property
    def owns_buffer(self):
        return self._owns_buffer

    @property
    def owns_pointer(self):
        return self._owns_pointer

    @property
    def is_owner(self):
        return self._owns_buffer and self._owns_pointer

    def _q(self, name):
        return int(getattr(self._lib, name)(self.pointer))

    slot_size = property(lambda self: self._q("st_Buffer_get_slot_size"))
    size = property(lambda self: self._q("st_Buffer_get_size"))
    capacity = property(lambda self: self._q("st_Buffer_get_capacity"))
    num_objects = property(lambda self: self._q("st_Buffer_get_num_of_objects"))
    max_num_objects = property(lambda self: self._q("st_Buffer_get_max_num_of_objects"))
    num_slots = property(lambda self: self._q("st_Buffer_get_num_of_slots"))
    max_num_slots = property(lambda self: self._q("st_Buffer_get_max_num_of_slots"))
    num_dataptrs = property(lambda self: self._q("st_Buffer_get_num_of_dataptrs"))
    max_num_dataptrs = property(lambda self: self._q("st_Buffer_get_max_num_of_dataptrs"))
    num_garbage_ranges = property(lambda self: self._q("st_Buffer_get_num_of_garbage_ranges"))
    max_num_garbage_ranges = property(
        lambda self: self._q("st_Buffer_get_max_num_of_garbage_ranges"))
    header_size = property(lambda self: self._q("st_Buffer_get_header_size"))
    data_begin_addr = property(lambda self: self._q("st_Buffer_get_data_begin_addr"))
    data_end_addr = property(lambda self: self._q("st_Buffer_get_data_end_addr"))

    @property
    def needs_remapping(self):
        return bool(self._lib.st_Buffer_needs_remapping(self.pointer))

    @property
    def ptr_data_begin(self):
        return C.cast(self.data_begin_addr, C.POINTER(C.c_ubyte))

    @property
    def ptr_data_end(self):
        return C.cast(self.data_end_addr, C.POINTER(C.c_ubyte))

    # ------------------------------------------------------------ changes
    def _status(self, st, what):
        self._last_status = int(st)
        if self._last_status != 0:
            raise RuntimeError(f"unsuccessful {what} op; status:{self._last_status}")
        return self

    def clear(self, clear_data=False):
        return self._status(self._lib.st_Buffer_clear(self.pointer, bool(clear_data)), "clear")

    def refresh(self):
        """Bring the C-side copy of a Python buffer up to date (the
        structure must be unchanged); otherwise the reference's refresh."""
        if self._cbuffer is not None and self._handle is not None:
            self._handle.refresh(self._cbuffer)
            return self._status(0, "refresh")
        return self._status(self._lib.st_Buffer_refresh(self.pointer), "refresh")

    def remap(self):
        return self._status(self._lib.st_Buffer_remap(self.pointer), "remap")

    def write_to_file(self, path_to_file, normalized_base_addr=None):
        if not path_to_file:
            self._last_status = -1
            raise RuntimeError("illegal path supplied")
        p = str(path_to_file).encode()
        if normalized_base_addr is not None and normalized_base_addr > 0:
            st = self._lib.st_Buffer_write_to_file_normalized_addr(self.pointer, p,
                                                                     int(normalized_base_addr))
        else:
            st = self._lib.st_Buffer_write_to_file(self.pointer, p)
        return self._status(st, "write_to_file")

    def read_from_file(self, path_to_file):
        if path_to_file:
            self._status(self._lib.st_Buffer_read_from_file(self.pointer,
                                                            str(path_to_file).encode()),
                         "read_from_file")
        return self

    def reserve_capacity(self, capacity):
        if capacity is not None and capacity >= 0:
            self._status(self._lib.st_Buffer_reserve_capacity(self.pointer, int(capacity)),
                         "reserve capacity")
        return self

    def reserve(self, max_num_objects, max_num_slots, max_num_dataptrs,
                max_num_garbage_ranges):
        return self._status(self._lib.st_Buffer_reserve(
            self.pointer, int(max_num_objects), int(max_num_slots), int(max_num_dataptrs),
            int(max_num_garbage_ranges)), "reserve")

    def reset(self, max_num_objects=None, max_num_slots=None, max_num_dataptrs=None,
              max_num_garbage_ranges=None):
        if (max_num_objects, max_num_slots, max_num_dataptrs,
                max_num_garbage_ranges) == (None, None, None, None):
            return self._status(self._lib.st_Buffer_reset(self.pointer), "reset")
        return self._status(self._lib.st_Buffer_reset_detailed(
            self.pointer,
            int(self.max_num_objects if max_num_objects is None else max_num_objects),
            int(self.max_num_slots if max_num_slots is None else max_num_slots),
            int(self.max_num_dataptrs if max_num_dataptrs is None else max_num_dataptrs),
            int(max_num_garbage_ranges or 0)), "reset")

    def image(self) -> np.ndarray:
        """A copy of the buffer's CObjects image."""
        n = self.size
        data = self._lib.st_Buffer_get_const_data_begin(self.pointer)
        return np.ctypeslib.as_array(C.cast(data, C.POINTER(C.c_uint64)), shape=(n // 8,)).copy()


class AssignAddressItem(_Element):
    """One address assignment (buffer.py:69-78); element indices default
    to 1, as in the reference."""

    _typeid = TYPE_ASSIGN_ADDRESS_ITEM
    _fields = (
        ("dest_buffer_id", "u"), ("src_buffer_id", "u"),
        ("dest_elem_type_id", "u"), ("src_elem_type_id", "u"),
        ("dest_elem_index", "u"), ("src_elem_index", "u"),
        ("dest_pointer_offset", "u"), ("src_pointer_offset", "u"),
    )
    _default_dest_elem_index = 1
    _default_src_elem_index = 1

    def key(self):
        return tuple(int(getattr(self, name)) for name, _ in self._fields)


class AddressAssignments:
    """The assignment items of one job, in the order they were added."""

    FIELDS = tuple(name for name, _ in AssignAddressItem._fields)

    def __init__(self):
        self.items = []

    @classmethod
    def make(cls, item=None, **fields):
        """An item from an AssignAddressItem or from all eight fields."""
        if item is not None:
            if not isinstance(item, AssignAddressItem):
                raise TypeError("item must be an AssignAddressItem")
            return item
        if any(fields.get(f) is None for f in cls.FIELDS):
            raise ValueError("unable to add AssignAddressItem given by these parameters")
        return AssignAddressItem(**{f: int(fields[f]) for f in cls.FIELDS})

    def add(self, item):
        k = item.key()
        for it in self.items:
            if it.key() == k:
                return it
        self.items.append(item)
        return item

    def index_of(self, item):
        k = item.key()
        for i, it in enumerate(self.items):
            if it.key() == k:
                return i
        return None

    def between(self, dest_buffer_id, src_buffer_id):
        return [it for it in self.items
                if it.dest_buffer_id == dest_buffer_id and it.src_buffer_id == src_buffer_id]

    def perform(self, handles: dict, cbuffers: dict, dest_buffer_id=None, src_buffer_id=None):
        """Carry out the items (all, or those between the two buffers);
        ``handles`` / ``cbuffers`` map buffer ids to the job's C-side copies
        and Python buffers.  Returns the destination buffer ids written."""
        written = set()
        for it in self.items:
            if dest_buffer_id is not None and (it.dest_buffer_id != dest_buffer_id or
                                               it.src_buffer_id != src_buffer_id):
                continue
            src, dst = handles.get(it.src_buffer_id), cbuffers.get(it.dest_buffer_id)
            if src is None or dst is None:
                raise RuntimeError(f"assignment between unknown buffers {it.dest_buffer_id} "
                                   f"<- {it.src_buffer_id}")
            b, t, s = src.object_info(int(it.src_elem_index))
            off = int(it.src_pointer_offset)
            if t != it.src_elem_type_id or s < off + 8 or (b + off) % 8:
                raise RuntimeError(f"source object {it.src_elem_index} of buffer "
                                   f"{it.src_buffer_id} does not match the item")
            di, doff = int(it.dest_elem_index), int(it.dest_pointer_offset)
            if not 0 <= di < len(dst.objects):
                raise RuntimeError(f"destination object {di} outside buffer {it.dest_buffer_id}")
            obj = dst.objects[di]
            nstruct = obj.words.size if not obj.ptr_fields else min(
                int(obj.words[f]) for f in obj.ptr_fields)
            if obj.typeid != it.dest_elem_type_id or doff % 8 or doff + 8 > 8 * nstruct:
                raise RuntimeError(f"destination object {di} of buffer {it.dest_buffer_id} "
                                   f"does not match the item")
            obj.words[doff // 8] = np.uint64(b + off)
            obj.links = [(f, tgt) for f, tgt in obj.links if f != doff // 8]
            dst.touch()
            written.add(int(it.dest_buffer_id))
        return written
