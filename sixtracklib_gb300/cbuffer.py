"""CObjects buffer images, readable and writable from Python.

SixTrackLib stores lattices and particle sets as "CObjects" buffers: a flat,
8-byte-slot image with a header and four sections (slots, objects, dataptrs,
garbage).  The layout is fixed by the reference
(sixtracklib/common/buffer/managed_buffer_minimal.h:396-770,
buffer/buffer_object.h:24-30, buffer/managed_buffer_remap.h:180-644):

* header: u64 words ``[base_addr, buffer_size, header_size, slots_addr,
  objects_addr, dataptrs_addr, garbage_addr, 0]``;
* every section: ``[section_size_bytes, num_entities, entries...]``;
* an object entry: ``{begin_addr, type_id, size_bytes}``;
* a dataptrs entry: the absolute address of a pointer field inside an object,
  whose stored value is itself an absolute address into the slots section.

Addresses are absolute with respect to ``base_addr``; remapping a buffer to a
new base shifts all of them.  This module keeps objects in a base-independent
form (pointer fields hold word offsets relative to the object start) and
produces an absolute image on demand, so images written here load in the
reference (``NS(Buffer_new_from_file)``) and images written by the reference
or its Python layer (``cobjects``) load here.
"""

from __future__ import annotations

import os
from dataclasses import dataclass, field

import numpy as np

SLOT = 8
HEADER_WORDS = 8
DEFAULT_BASE = 4096
TYPE_SC_INTERPOLATED_PROF = 257
TYPE_TRICUB = 261


@dataclass
class CObject:
    """One stored object: its type id, its words (struct followed by the
    arrays its pointer fields reference) and the word indices of the pointer
    fields, whose entries in ``words`` are word offsets from the object start."""

    typeid: int
    words: np.ndarray
    ptr_fields: list = field(default_factory=list)
    # (field index, object index): plain address fields that hold the
    # absolute address of another object of the same buffer (not dataptrs:
    # the reference leaves them to its TrackJob's address assignment)
    links: list = field(default_factory=list)

    @property
    def nbytes(self) -> int:
        return int(self.words.size) * SLOT

    def reals(self) -> np.ndarray:
        return self.words.view(np.float64)

    def ints(self) -> np.ndarray:
        return self.words.view(np.int64)


class CBuffer:
    """A CObjects buffer held as a list of :class:`CObject`.

    Mirrors the role of ``cobjects.CBuffer`` used by the reference Python
    bindings (python/sixtracklib/trackjob.py:1285-1445), restricted to what
    the tracking path needs: add objects, read them back, serialise.
    """

    def __init__(self):
        self.objects: list[CObject] = []
        self.typeids: dict[int, type] = {}
        self._image_cache = None

    # ------------------------------------------------------------ building
    def add_object(self, typeid: int, struct_words, arrays=(), links=()) -> int:
        """Append an object.

        ``struct_words``: the fixed struct as u64 words; pointer fields may
        hold anything.  ``arrays``: ``[(field_index, values)]`` -- each array
        is appended after the struct (8-byte aligned) and the pointer field at
        ``field_index`` is made to reference it.  ``links``: ``[(field_index,
        object_index)]`` -- the field receives that object's absolute address
        in every image.  Returns the object index.
        """
        sw = _as_words(struct_words)
        parts = [sw]
        ptrs = []
        off = sw.size
        for fidx, values in arrays:
            vw = _as_words(values)
            sw[fidx] = off
            ptrs.append(int(fidx))
            parts.append(vw)
            off += vw.size
        words = np.concatenate(parts) if len(parts) > 1 else sw.copy()
        self.objects.append(CObject(int(typeid), words, ptrs,
                                    [(int(f), int(t)) for f, t in links]))
        self._image_cache = None
        return len(self.objects) - 1

    def add_raw(self, obj: CObject) -> int:
        self.objects.append(CObject(obj.typeid, obj.words.copy(), list(obj.ptr_fields),
                                    list(obj.links)))
        self._image_cache = None
        return len(self.objects) - 1

    def touch(self):
        """Invalidate the cached image after objects were edited in place."""
        self._image_cache = None

    @property
    def n_objects(self) -> int:
        return len(self.objects)

    num_objects = n_objects  # the reference's Buffer spells it so

    @property
    def size(self) -> int:
        """Size of the buffer's image in bytes."""
        return int(self.to_image().nbytes)

    def get_object(self, index: int, cls=None):
        """Object ``index`` decoded as ``cls`` (default: the class registered
        for its type id), or the raw CObject."""
        obj = self.objects[index]
        cls = cls if cls is not None else self.typeids.get(obj.typeid)
        if cls is not None and hasattr(cls, "_from_cobject"):
            return cls._from_cobject(obj, self, index)
        return obj

    # ------------------------------------------------------- serialisation
    def to_image(self, base: int = DEFAULT_BASE) -> np.ndarray:
        """Absolute CObjects image as a u64 array (cached until changed)."""
        if self._image_cache is not None and self._image_cache[0] == base:
            return self._image_cache[1]
        nslots = sum(o.words.size for o in self.objects)
        ndp = sum(len(o.ptr_fields) for o in self.objects)
        nobj = len(self.objects)
        slots_w = HEADER_WORDS
        objs_w = slots_w + 2 + nslots
        dp_w = objs_w + 2 + 3 * nobj
        gb_w = dp_w + 2 + ndp
        total_w = gb_w + 2
        img = np.zeros(total_w, dtype=np.uint64)
        img[0:7] = [
            base,
            total_w * SLOT,
            HEADER_WORDS * SLOT,
            base + slots_w * SLOT,
            base + objs_w * SLOT,
            base + dp_w * SLOT,
            base + gb_w * SLOT,
        ]
        img[slots_w] = (objs_w - slots_w) * SLOT
        img[slots_w + 1] = nslots
        img[objs_w] = (dp_w - objs_w) * SLOT
        img[objs_w + 1] = nobj
        img[dp_w] = (gb_w - dp_w) * SLOT
        img[dp_w + 1] = ndp
        img[gb_w] = 2 * SLOT
        img[gb_w + 1] = 0
        starts = np.cumsum([0] + [o.words.size for o in self.objects]) + (slots_w + 2)
        pos = slots_w + 2
        k = 0
        for i, o in enumerate(self.objects):
            n = o.words.size
            seg = o.words.copy()
            for f in o.ptr_fields:
                seg[f] = base + (pos + int(o.words[f])) * SLOT
                img[dp_w + 2 + k] = base + (pos + f) * SLOT
                k += 1
            for f, t in o.links:
                seg[f] = base + int(starts[t]) * SLOT
            img[pos : pos + n] = seg
            e = objs_w + 2 + 3 * i
            img[e] = base + pos * SLOT
            img[e + 1] = o.typeid
            img[e + 2] = n * SLOT
            pos += n
        self._image_cache = (base, img)
        return img

    def to_bytes(self, base: int = DEFAULT_BASE) -> bytes:
        return self.to_image(base).tobytes()

    def tofile(self, path):
        with open(path, "wb") as f:
            f.write(self.to_bytes())

    @classmethod
    def from_bytes(cls, data) -> "CBuffer":
        img = np.frombuffer(bytes(data), dtype=np.uint64).copy()
        return cls.from_image(img)

    @classmethod
    def fromfile(cls, path) -> "CBuffer":
        with open(os.fspath(path), "rb") as f:
            return cls.from_bytes(f.read())

    @classmethod
    def from_image(cls, img: np.ndarray) -> "CBuffer":
        img = np.asarray(img, dtype=np.uint64)
        base = int(img[0])
        size = int(img[1])
        if size % SLOT or size // SLOT > img.size:
            raise ValueError("CObjects image: inconsistent buffer size")

        def w(addr):
            off = int(addr) - base
            if off < 0 or off % SLOT or off // SLOT >= img.size:
                raise ValueError("CObjects image: address outside the buffer")
            return off // SLOT

        objs_w = w(img[4])
        nobj = int(img[objs_w + 1])
        dp_w = w(img[5])
        ndp = int(img[dp_w + 1])
        dptrs = sorted(w(a) for a in img[dp_w + 2 : dp_w + 2 + ndp])
        out = cls()
        starts = []
        for i in range(nobj):
            e = objs_w + 2 + 3 * i
            b = w(img[e])
            n = int(img[e + 2]) // SLOT
            starts.append((b, n, int(img[e + 1])))
        di = 0
        for b, n, t in starts:
            words = img[b : b + n].copy()
            ptrs = []
            while di < len(dptrs) and dptrs[di] < b:
                di += 1
            j = di
            while j < len(dptrs) and dptrs[j] < b + n:
                f = dptrs[j] - b
                tgt = w(img[dptrs[j]]) - b
                if 0 <= tgt <= n:
                    words[f] = tgt
                    ptrs.append(f)
                j += 1
            out.objects.append(CObject(t, words, ptrs))
        # interpolated space charge (type 257): field 6 addresses the line
        # density object of the same buffer when it is linked; TriCub (261):
        # field 7 its TriCubData likewise
        begin_index = {b: i for i, (b, _, _) in enumerate(starts)}
        base_w = {base + b * SLOT: i for b, i in begin_index.items()}
        for o in out.objects:
            for typeid, f in ((TYPE_SC_INTERPOLATED_PROF, 6), (TYPE_TRICUB, 7)):
                if o.typeid == typeid and o.words.size > f:
                    tgt = base_w.get(int(o.words[f]))
                    if tgt is not None:
                        o.links.append((f, tgt))
        return out


def _as_words(values) -> np.ndarray:
    a = np.asarray(values)
    if a.dtype == np.float64:
        return a.astype(np.float64, copy=True).view(np.uint64).reshape(-1)
    if a.dtype.kind in "iu":
        return a.astype(np.int64, copy=True).view(np.uint64).reshape(-1)
    if a.dtype == object or a.dtype.kind == "f":
        return np.asarray(a, dtype=np.float64).view(np.uint64).reshape(-1).copy()
    raise TypeError(f"cannot store dtype {a.dtype} in a CObjects buffer")
