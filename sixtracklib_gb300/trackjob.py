"""TrackJob / CudaTrackJob over the engine's C ABI.

Mirrors python/sixtracklib/trackjob.py:1285-1700 (constructor arguments,
``track_until`` / ``track_elem_by_elem`` / ``track_line``, ``collect*`` /
``push*``, output properties, RuntimeError on a non-zero track status).
Buffers may be :class:`~sixtracklib_gb300.cbuffer.CBuffer` objects or
containers holding one (``Elements``, ``ParticlesSet``, ``Particles``).

The job keeps the particle columns and the compiled lattice resident on the
GPU; ``collect_particles`` copies the columns back into the caller's Python
buffer in place, ``collect_output`` refreshes :attr:`output`.
"""

from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native
from .cbuffer import CBuffer
from .particles import TYPE_PARTICLE, Particles


def get_cbuffer_from_obj(obj) -> CBuffer:
    if isinstance(obj, CBuffer):
        return obj
    for attr in ("cbuffer", "_cbuffer"):
        cb = getattr(obj, attr, None)
        if isinstance(cb, CBuffer):
            return cb
    raise TypeError(f"cannot get a CObjects buffer from {type(obj).__name__}")


class _CBufferHandle:
    """A C-side st_Buffer holding a copy of a Python CBuffer image."""

    def __init__(self, cbuffer: CBuffer):
        lib = _native.load()
        img = cbuffer.to_image()
        self.ptr = lib.st_Buffer_new_on_data(img.ctypes.data, img.nbytes)
        if not self.ptr:
            raise RuntimeError("st_Buffer_new_on_data failed: " + _native.last_error())

    def image(self) -> np.ndarray:
        lib = _native.load()
        n = lib.st_Buffer_get_size(self.ptr)
        data = lib.st_Buffer_get_const_data_begin(self.ptr)
        return np.ctypeslib.as_array(C.cast(data, C.POINTER(C.c_uint64)), shape=(n // 8,)).copy()

    def free(self):
        if self.ptr:
            _native.load().st_Buffer_delete(self.ptr)
            self.ptr = None


class TrackJob:
    def __init__(self, beam_elements_buffer, particles_buffer, until_turn_elem_by_elem=0,
                 arch="cuda", device_id=None, device=None, output_buffer=None,
                 config_str=None, particle_set_indices=None):
        self._lib = _native.load()
        self.ptr_st_track_job = None
        self._arch = (arch or "cuda").lower()
        self._particles_buffer = get_cbuffer_from_obj(particles_buffer)
        self._beam_elements_buffer = get_cbuffer_from_obj(beam_elements_buffer)
        self._c_particles = _CBufferHandle(self._particles_buffer)
        self._c_elements = _CBufferHandle(self._beam_elements_buffer)
        self._c_output = None
        self._output_buffer = None
        self._user_output = output_buffer
        self._last_status = 0
        cfg = config_str or ""
        dev = device if device is not None else device_id
        if dev is not None:
            d = str(dev)
            d = d.split(".")[-1] if "." in d else d
            cfg = (cfg + "\n" if cfg else "") + f"device={d}"
        if output_buffer is not None:
            self._c_output = _CBufferHandle(get_cbuffer_from_obj(output_buffer))
        if particle_set_indices is None:
            idx = [i for i, o in enumerate(self._particles_buffer.objects)
                   if o.typeid == TYPE_PARTICLE][:1]
        else:
            idx = list(particle_set_indices)
        self._pset_indices = idx
        arr = (C.c_uint64 * max(len(idx), 1))(*idx)
        self.ptr_st_track_job = self._lib.st_TrackJob_new_detailed(
            self._arch.encode(), self._c_particles.ptr, len(idx), arr, self._c_elements.ptr,
            self._c_output.ptr if self._c_output else None, int(until_turn_elem_by_elem),
            cfg.encode())
        if not self.ptr_st_track_job:
            raise RuntimeError("unable to create TrackJob: " + _native.last_error())
        if self._lib.st_TrackJob_has_output_buffer(self.ptr_st_track_job):
            self._refresh_output()

    def __del__(self):
        try:
            if self.ptr_st_track_job:
                self._lib.st_TrackJob_delete(self.ptr_st_track_job)
                self.ptr_st_track_job = None
            for h in (getattr(self, "_c_particles", None), getattr(self, "_c_elements", None),
                      getattr(self, "_c_output", None)):
                if h is not None:
                    h.free()
        except Exception:
            pass

    # ---------------------------------------------------------- properties
    @property
    def last_status(self):
        return self._last_status

    last_track_status = last_status

    @property
    def arch(self):
        return self._arch

    @property
    def arch_str(self):
        return self._arch

    def type_str(self):
        return self._lib.st_TrackJob_get_type_str(self.ptr_st_track_job).decode()

    @property
    def particles_buffer(self):
        return self._particles_buffer

    @property
    def beam_elements_buffer(self):
        return self._beam_elements_buffer

    @property
    def output_buffer(self):
        return self._output_buffer

    @property
    def output(self):
        return self._output_buffer

    @property
    def has_output_buffer(self):
        return bool(self._lib.st_TrackJob_has_output_buffer(self.ptr_st_track_job))

    @property
    def has_elem_by_elem_output(self):
        return bool(self._lib.st_TrackJob_has_elem_by_elem_output(self.ptr_st_track_job))

    @property
    def has_beam_monitor_output(self):
        return bool(self._lib.st_TrackJob_has_beam_monitor_output(self.ptr_st_track_job))

    @property
    def elem_by_elem_output_offset(self):
        return int(self._lib.st_TrackJob_get_elem_by_elem_output_buffer_offset(self.ptr_st_track_job))

    @property
    def beam_monitor_output_offset(self):
        return int(self._lib.st_TrackJob_get_beam_monitor_output_buffer_offset(self.ptr_st_track_job))

    @property
    def num_beam_monitors(self):
        return int(self._lib.st_TrackJob_get_num_beam_monitors(self.ptr_st_track_job))

    @property
    def requires_collecting(self):
        return True

    # ------------------------------------------------------------ tracking
    def _check(self, st, what):
        self._last_status = int(st)
        if st != 0:
            msg = _native.last_error()
            raise RuntimeError(f"{what} failed with status {st}" + (f": {msg}" if msg else ""))
        return st

    def track(self, until_turn):
        return self.track_until(until_turn)

    def track_until(self, until_turn):
        return self._check(self._lib.st_TrackJob_track_until(self.ptr_st_track_job, int(until_turn)),
                           "track_until")

    def track_elem_by_elem(self, until_turn):
        return self._check(
            self._lib.st_TrackJob_track_elem_by_elem(self.ptr_st_track_job, int(until_turn)),
            "track_elem_by_elem")

    def track_line(self, begin_idx, end_idx, finish_turn=False):
        return self._check(self._lib.st_TrackJob_track_line(
            self.ptr_st_track_job, int(begin_idx), int(end_idx), bool(finish_turn)), "track_line")

    # ----------------------------------------------------- collect / push
    def collect(self):
        self.collect_particles()
        self.collect_output()

    def collect_particles(self):
        self._lib.st_TrackJob_collect_particles(self.ptr_st_track_job)
        for i in self._pset_indices:
            cols = _c_columns(self._lib, self._c_particles.ptr, i)
            self._particles_buffer.get_object(i).set_block(cols)
        self._particles_buffer.touch()
        return self

    def collect_beam_elements(self):
        return self

    def collect_output(self):
        if self.has_output_buffer:
            self._lib.st_TrackJob_collect_output(self.ptr_st_track_job)
            self._refresh_output()
        return self

    def push_particles(self):
        for i in self._pset_indices:
            blk = self._particles_buffer.get_object(i).block
            _c_columns(self._lib, self._c_particles.ptr, i, write=blk)
        self._lib.st_TrackJob_push_particles(self.ptr_st_track_job)
        return self

    def push_beam_elements(self):
        self._lib.st_TrackJob_push_beam_elements(self.ptr_st_track_job)
        return self

    def _refresh_output(self):
        ptr = self._lib.st_TrackJob_get_output_buffer(self.ptr_st_track_job)
        n = self._lib.st_Buffer_get_size(ptr)
        data = self._lib.st_Buffer_get_const_data_begin(ptr)
        img = np.ctypeslib.as_array(C.cast(data, C.POINTER(C.c_uint64)), shape=(n // 8,)).copy()
        self._output_buffer = CBuffer.from_image(img)
        self._output_buffer.typeids[TYPE_PARTICLE] = Particles

    def output_particles(self, index) -> Particles:
        """Particles object ``index`` of the output buffer."""
        return self._output_buffer.get_object(index)


class _StParticles(C.Structure):
    _fields_ = [("num_particles", C.c_int64)] + [(f"c{i}", C.c_void_p) for i in range(21)]


def _c_columns(lib, c_buffer, index, write=None):
    """Read (or overwrite) the 21 x n columns of Particles object `index` of a
    C-side st_Buffer."""
    ptr = lib.st_Particles_buffer_get_particles(c_buffer, int(index))
    if not ptr:
        raise RuntimeError(f"object {index} is not a Particles object")
    sp = _StParticles.from_address(ptr)
    n = int(sp.num_particles)
    out = np.empty((21, n), dtype=np.uint64)
    for c in range(21):
        col = np.ctypeslib.as_array(C.cast(getattr(sp, f"c{c}"), C.POINTER(C.c_uint64)), shape=(n,))
        if write is not None:
            col[:] = np.asarray(write[c]).view(np.uint64)
        else:
            out[c] = col
    return out


class CudaTrackJob(TrackJob):
    """cuda/track_job.h:42-66 / python/sixtracklib/cuda.py:565: a TrackJob
    bound to a CUDA node id ("platform.device")."""

    def __init__(self, beam_elements_buffer, particles_buffer, until_turn_elem_by_elem=0,
                 node_id_str=None, output_buffer=None, config_str=None, **kw):
        super().__init__(beam_elements_buffer, particles_buffer, until_turn_elem_by_elem,
                         arch="cuda", device=node_id_str, output_buffer=output_buffer,
                         config_str=config_str, **kw)
