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
    """The view of a stored buffer that ``TrackJob.stored_buffer`` returns
    (buffer.py:92-200): the job's C-side copy (``pointer``), its object
    count and size, and the Python buffer it copies (``cbuffer``)."""

    maps_to_cbuffer = True

    def __init__(self, cbuffer: CBuffer, handle: CBufferHandle):
        self.cbuffer = cbuffer
        self._handle = handle

    @property
    def pointer(self):
        return self._handle.ptr

    @property
    def num_objects(self):
        return int(self._handle._lib.st_Buffer_get_num_of_objects(self._handle.ptr))

    @property
    def size(self):
        return int(self._handle._lib.st_Buffer_get_size(self._handle.ptr))


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
