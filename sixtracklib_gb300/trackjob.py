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
import warnings

import numpy as np

from . import _native
from .beam_elements import TYPE_BEAM_MONITOR
from .buffer import (ARCH_BEAM_ELEMENTS_BUFFER_ID, ARCH_ILLEGAL_BUFFER_ID,
                     ARCH_MIN_USER_DEFINED_BUFFER_ID, ARCH_PARTICLES_BUFFER_ID,
                     AddressAssignments, Buffer, CBufferHandle)
from .cbuffer import CBuffer
from .particles import TYPE_PARTICLE, Particles, ParticlesSet


def get_cbuffer_from_obj(obj) -> CBuffer:
    from .buffer import get_cbuffer_from_obj as find

    cb = find(obj)
    if cb is None:
        raise TypeError(f"cannot get a CObjects buffer from {type(obj).__name__}")
    return cb


_CBufferHandle = CBufferHandle


class TrackJob:
    def __init__(self, beam_elements_buffer, particles_buffer, until_turn_elem_by_elem=0,
                 arch="cuda", device_id=None, device=None, output_buffer=None,
                 config_str=None, particle_set_indices=None):
        self._lib = _native.load()
        self.ptr_st_track_job = None
        self._stored = {}  # buffer id -> (CBuffer, CBufferHandle, owned)
        self._next_stored_id = ARCH_MIN_USER_DEFINED_BUFFER_ID
        self._assign = AddressAssignments()
        self._assigned = False
        self._setup(beam_elements_buffer, particles_buffer, until_turn_elem_by_elem, arch,
                    device_id, device, output_buffer, config_str, particle_set_indices)

    def _setup(self, beam_elements_buffer, particles_buffer, until_turn_elem_by_elem, arch,
               device_id, device, output_buffer, config_str, particle_set_indices):
        self._ctor = (arch, device_id, device, config_str)
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
        # set-up writes into the beam elements (monitors' particle-id ranges)
        self._c_elements.pull_into(self._beam_elements_buffer)
        if self._lib.st_TrackJob_has_output_buffer(self.ptr_st_track_job):
            self._refresh_output()

    def _release_job(self):
        if self.ptr_st_track_job:
            self._lib.st_TrackJob_delete(self.ptr_st_track_job)
            self.ptr_st_track_job = None
        for attr in ("_c_particles", "_c_elements", "_c_output"):
            h = getattr(self, attr, None)
            if h is not None:
                h.free()
            setattr(self, attr, None)

    def __del__(self):
        try:
            self._release_job()
            for _cb, h, _own in getattr(self, "_stored", {}).values():
                h.free()
        except Exception:
            pass

    def reset(self, beam_elements_buffer, particles_buffer, until_turn_elem_by_elem=0,
              output_buffer=None):
        """Re-create the job on new buffers (trackjob.py:2044-2100), keeping
        the arch, device and configuration; stored buffers and assignment
        items are kept, and assignments already carried out are carried out
        again on the new beam elements."""
        arch, device_id, device, config_str = self._ctor
        self._release_job()
        self._setup(beam_elements_buffer, particles_buffer, until_turn_elem_by_elem, arch,
                    device_id, device, output_buffer, config_str, None)
        if self._assigned:
            self.assign_all_addresses()
        return self

    # ---------------------------------------------------------- properties
    @property
    def last_status(self):
        return self._last_status

    last_track_status = last_status

    @property
    def last_status_success(self):
        return self._last_status == 0

    last_track_status_success = last_status_success

    @property
    def is_in_debug_mode(self):
        """Debug mode (track/track_job_base.h:182-189): every tracking call
        first validates its inputs and records the outcome in the debug
        register."""
        return bool(self._lib.st_TrackJobNew_is_in_debug_mode(self.ptr_st_track_job))

    def _status(self, st, what):
        """raise_error_if_status_not_success (control.py:181-189)."""
        self._last_status = int(st)
        if st != 0:
            raise RuntimeError(f"unsuccessful {what} op; status:{st}")
        return self

    def enable_debug_mode(self):
        return self._status(self._lib.st_TrackJobNew_enable_debug_mode(self.ptr_st_track_job),
                            "enable debug mode")

    def disable_debug_mode(self):
        return self._status(self._lib.st_TrackJobNew_disable_debug_mode(self.ptr_st_track_job),
                            "disable debug mode")

    def collect_debug_flag(self):
        """Reads the debug register back (fails outside debug mode)."""
        return self._status(self._lib.st_TrackJobNew_collect_debug_flag(self.ptr_st_track_job),
                            "debug flag collection")

    @property
    def debug_register(self):
        return int(self._lib.st_TrackJobNew_get_debug_register(self.ptr_st_track_job))

    @property
    def is_collecting_particles(self):
        return bool(self._lib.st_TrackJob_is_collecting_particles(self.ptr_st_track_job))

    @property
    def num_particle_sets(self):
        return len(self._pset_indices)

    @property
    def owns_output_buffer(self):
        return bool(self._lib.st_TrackJob_owns_output_buffer(self.ptr_st_track_job))

    @property
    def arch(self):
        return self._arch

    @property
    def arch_str(self):
        return self._arch

    def type_str(self):
        return self._lib.st_TrackJob_get_type_str(self.ptr_st_track_job).decode()

    def type(self):
        """The architecture id of the job: 3, SIXTRL_ARCHITECTURE_CUDA
        (trackjob.py:1622-1632)."""
        return int(self._lib.st_TrackJob_get_type_id(self.ptr_st_track_job))

    @property
    def arch_id(self):
        return self.type()

    # ---------------------------------- nodes (trackjob.py:1215-1290)
    @staticmethod
    def enabled_archs():
        """The architectures this engine tracks on: CUDA only (the reference
        lists its compiled modules plus "cpu")."""
        return ["cuda"]

    @staticmethod
    def num_available_nodes(arch_str=None, env_var_name=None, filter_str=None):
        """CUDA devices this process can use for arch "cuda" (the reference
        counts OpenCL nodes only and answers 0 otherwise); 0 for other archs."""
        if arch_str is None or arch_str.strip().lower() != "cuda":
            return 0
        return int(_native.load().st_CudaTrackJob_get_num_available_nodes())

    @staticmethod
    def num_all_nodes(arch_str=None):
        return TrackJob.num_available_nodes(arch_str)

    @staticmethod
    def print_nodes(arch_str, all=False, filter_str=None, env_var_name=None):
        """Print the CUDA devices (node index = device index) for arch "cuda"."""
        n = TrackJob.num_available_nodes(arch_str)
        if n == 0:
            print(f"no nodes available for arch {arch_str!r}")
            return
        try:
            import torch

            names = [torch.cuda.get_device_name(k) for k in range(n)]
        except Exception:  # the names are cosmetic; the count comes from the driver
            names = ["CUDA device"] * n
        for k, name in enumerate(names):
            print(f"cuda node {k}: {name}")

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
        """The output buffer as a particle-set container (trackjob.py:571)."""
        return ParticlesSet(self._output_buffer) if self._output_buffer is not None else None

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

    # --------------- TrackJobBaseNew names (python/sixtracklib/trackjob.py)
    @property
    def pointer(self):
        return self.ptr_st_track_job

    @property
    def total_num_particles(self):
        return int(self._lib.st_TrackJob_get_total_num_particles_in_sets(self.ptr_st_track_job))

    @property
    def collecting_flags(self):
        return int(self._lib.st_TrackJob_get_collect_flags(self.ptr_st_track_job))

    @property
    def is_collecting_beam_elements(self):
        return bool(self._lib.st_TrackJob_is_collecting_beam_elements(self.ptr_st_track_job))

    @property
    def is_collecting_output(self):
        return bool(self._lib.st_TrackJob_is_collecting_output(self.ptr_st_track_job))

    @property
    def has_config_str(self):
        return bool(self._lib.st_TrackJob_has_config_str(self.ptr_st_track_job))

    @property
    def has_elem_by_elem_config(self):
        return bool(self._lib.st_TrackJob_has_elem_by_elem_config(self.ptr_st_track_job))

    @property
    def has_beam_monitors(self):
        return bool(self._lib.st_TrackJob_has_beam_monitors(self.ptr_st_track_job))

    @property
    def num_elem_by_elem_turn(self):
        """The number of turns the elem-by-elem output stores (the reference's
        property returns the output's buffer offset under this name)."""
        return int(self._lib.st_TrackJob_get_num_elem_by_elem_turns(self.ptr_st_track_job))

    elem_by_elem_output_buffer_offset = property(lambda self: self.elem_by_elem_output_offset)
    beam_monitor_output_buffer_offset = property(lambda self: self.beam_monitor_output_offset)
    # the job keeps its device data as the reference's CUDA job keeps its
    # arguments, bound to its node as the reference's controller is
    uses_arguments = property(lambda self: self.ptr_st_track_job is not None)
    uses_controller = property(lambda self: self.ptr_st_track_job is not None)

    def collect_particle_addresses(self):
        """The device addresses of the particle sets (the reference collects
        them from its device argument; here they are formed on the host)."""
        return self.fetch_particle_addresses()

    # deprecated spellings of the reference (DeprecationWarning, then the call)
    def _deprecated(self, old, new):
        warnings.warn(f"{old}() is deprecated; use {new}() instead", DeprecationWarning,
                      stacklevel=3)
        return getattr(self, new)()

    def collectParticles(self):  # noqa: N802
        return self._deprecated("collectParticles", "collect_particles")

    def collectBeamElements(self):  # noqa: N802
        return self._deprecated("collectBeamElements", "collect_beam_elements")

    def collectOutput(self):  # noqa: N802
        return self._deprecated("collectOutput", "collect_output")

    def collectDebugFlag(self):  # noqa: N802
        return self._deprecated("collectDebugFlag", "collect_debug_flag")

    def collectParticlesAddresses(self):  # noqa: N802
        return self._deprecated("collectParticlesAddresses", "collect_particle_addresses")

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
        self._c_elements.pull_into(self._beam_elements_buffer)
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

    # ----------------------- particle addresses (trackjob.py, cuda.py:650-700)
    @property
    def can_fetch_particle_addresses(self):
        return bool(self._lib.st_TrackJob_can_fetch_particles_addr(self.ptr_st_track_job))

    @property
    def has_particle_addresses(self):
        return bool(self._lib.st_TrackJob_has_particles_addr(self.ptr_st_track_job))

    def fetch_particle_addresses(self):
        """Make the device addresses of the job's particle columns
        available (get_particle_addresses)."""
        self._last_status = int(
            self._lib.st_TrackJob_fetch_particle_addresses(self.ptr_st_track_job))
        if self._last_status != 0:
            raise RuntimeError("unable to fetch particle addresses")
        return self

    def clear_particle_addresses(self, particle_set_index=0):
        self._last_status = int(self._lib.st_TrackJob_clear_particle_addresses(
            self.ptr_st_track_job, int(particle_set_index)))
        return self

    def clear_all_particle_addresses(self):
        self._last_status = int(
            self._lib.st_TrackJob_clear_all_particle_addresses(self.ptr_st_track_job))
        return self

    def get_particle_addresses(self, particle_set_index=0):
        """A copy of the st_ParticlesAddr of particle set
        ``particle_set_index`` (its object index in the particles buffer):
        ``num_particles`` and the device address of each column; None when
        not fetched or not tracked by this job."""
        ptr = self._lib.st_TrackJob_particle_addresses(self.ptr_st_track_job,
                                                       int(particle_set_index))
        if not ptr:
            return None
        out = st_ParticlesAddr()
        C.memmove(C.addressof(out), ptr, C.sizeof(st_ParticlesAddr))
        return out

    def _push_output(self):
        """Send the host output buffer to the device copy (trackjob.py:1582)."""
        self._lib.st_TrackJob_push_output(self.ptr_st_track_job)
        return self

    def push_beam_elements(self):
        """Send the beam elements as they are now (edits made after the job
        was created included) and recompile the lattice."""
        self._c_elements.refresh(self._beam_elements_buffer)
        self._lib.st_TrackJob_push_beam_elements(self.ptr_st_track_job)
        return self

    # ---------------------------------- stored buffers (trackjob.py:2200-2290)
    def add_stored_buffer(self, cbuffer=None, size=None, ptr_c_buffer=None,
                          take_ownership=False, delete_ptr_after_move=False):
        """Keep a buffer with the job (for example line-density tables that
        beam elements point at); returns its id (>= 1024), or 0 when nothing
        usable was given.  ``size`` makes an empty buffer; a raw
        ``ptr_c_buffer`` is not supported (Python buffers only)."""
        if ptr_c_buffer is not None:
            raise NotImplementedError("stored buffers are Python CBuffers here")
        cb = get_cbuffer_from_obj(cbuffer) if cbuffer is not None else (
            CBuffer() if size is not None and size > 0 else None)
        if cb is None:
            return ARCH_ILLEGAL_BUFFER_ID
        bid = self._next_stored_id
        self._next_stored_id += 1
        self._stored[bid] = (cb, CBufferHandle(cb), cbuffer is None)
        return bid

    def remove_stored_buffer(self, buffer_id):
        entry = self._stored.pop(buffer_id, None)
        if entry is None:
            return -1
        entry[1].free()
        return 0

    @property
    def has_stored_buffers(self):
        return bool(self._stored)

    @property
    def num_stored_buffers(self):
        return len(self._stored)

    @property
    def min_stored_buffer_id(self):
        return min(self._stored) if self._stored else ARCH_ILLEGAL_BUFFER_ID

    @property
    def max_stored_buffer_id(self):
        return max(self._stored) if self._stored else ARCH_ILLEGAL_BUFFER_ID

    def owns_stored_buffer(self, buffer_id):
        return buffer_id in self._stored and self._stored[buffer_id][2]

    def stored_buffer_is_cbuffer(self, buffer_id):
        return buffer_id in self._stored

    def stored_buffer_cbuffer(self, buffer_id):
        if buffer_id not in self._stored:
            raise RuntimeError(f"Unable to retrieve CBuffer for buffer_id={buffer_id}")
        return self._stored[buffer_id][0]

    def stored_buffer(self, buffer_id):
        """A :class:`~sixtracklib_gb300.buffer.Buffer` view of the stored
        buffer (C-side copy and the Python buffer), or None."""
        entry = self._stored.get(buffer_id)
        return Buffer(cbuffer=entry[0], _handle=entry[1]) if entry is not None else None

    def ptr_stored_buffer(self, buffer_id):
        """The C-side st_Buffer of a stored buffer, or None."""
        entry = self._stored.get(buffer_id)
        return entry[1].ptr if entry is not None else None

    def push_stored_buffer(self, buffer_id):
        """Send the stored buffer's current contents (same structure)."""
        if buffer_id not in self._stored:
            raise RuntimeError(f"Unable to push stored buffer {buffer_id}")
        cb, h, _own = self._stored[buffer_id]
        h.refresh(cb)
        if any(it.src_buffer_id == buffer_id for it in self._assign.items) and self._assigned:
            self.push_beam_elements()  # the lattice holds copies of what it points at
        return self

    def collect_stored_buffer(self, buffer_id):
        """Bring the stored buffer up to date.  The engine writes a stored
        buffer only through BeamMonitors whose ``out_address`` was assigned
        from it: their turn-by-turn records (the job's own monitor output,
        the reference's layout) are copied into the assigned particle sets,
        as many particles as both hold."""
        if buffer_id not in self._stored:
            raise RuntimeError(f"Unable to collect stored buffer {buffer_id}")
        items = [it for it in self._assign.items
                 if it.src_buffer_id == buffer_id and
                 it.dest_buffer_id == ARCH_BEAM_ELEMENTS_BUFFER_ID and
                 it.dest_elem_type_id == TYPE_BEAM_MONITOR]
        if items and self._assigned and self.has_beam_monitor_output:
            self.collect_output()
            monitors = [i for i, o in enumerate(self._beam_elements_buffer.objects)
                        if o.typeid == TYPE_BEAM_MONITOR]
            cb, h, _own = self._stored[buffer_id]
            cb.typeids[TYPE_PARTICLE] = Particles
            for it in items:
                k = monitors.index(int(it.dest_elem_index))
                out = self.output_particles(self.beam_monitor_output_offset + k)
                dst = cb.get_object(int(it.src_elem_index))
                if not isinstance(dst, Particles):
                    continue
                n = min(dst.num_particles, out.num_particles)
                cols = dst.block.copy()
                cols[:, :n] = out.block[:, :n]
                dst.set_block(cols)
            cb.touch()
            h.refresh(cb)
        return self

    # ------------------------ address assignment (trackjob.py:1833-2035)
    def _buffers(self):
        """Sources (C-side copies by id) and destinations (Python buffers by
        id): the particles buffer can be a source only -- its C-side copy
        holds the tracked state."""
        handles = {ARCH_PARTICLES_BUFFER_ID: self._c_particles,
                   ARCH_BEAM_ELEMENTS_BUFFER_ID: self._c_elements}
        cbuffers = {ARCH_BEAM_ELEMENTS_BUFFER_ID: self._beam_elements_buffer}
        for bid, (cb, h, _own) in self._stored.items():
            handles[bid] = h
            cbuffers[bid] = cb
        return handles, cbuffers

    def add_assign_address_item(self, item=None, dest_elem_type_id=None, dest_buffer_id=None,
                                dest_elem_index=None, dest_pointer_offset=None,
                                src_elem_type_id=None, src_buffer_id=None, src_elem_index=None,
                                src_pointer_offset=None):
        """Add an item (an AssignAddressItem, or its eight fields); an item
        equal to one already added is not added twice.  Returns the item."""
        return self._assign.add(AddressAssignments.make(
            item, dest_elem_type_id=dest_elem_type_id, dest_buffer_id=dest_buffer_id,
            dest_elem_index=dest_elem_index, dest_pointer_offset=dest_pointer_offset,
            src_elem_type_id=src_elem_type_id, src_buffer_id=src_buffer_id,
            src_elem_index=src_elem_index, src_pointer_offset=src_pointer_offset))

    def _find(self, item, fields):
        try:
            it = AddressAssignments.make(item, **fields)
        except ValueError:
            return None
        i = self._assign.index_of(it)
        return None if i is None else self._assign.items[i]

    def has_assign_item(self, item=None, dest_buffer_id=None, src_buffer_id=None, index=None,
                        **fields):
        if item is None and index is not None:
            return 0 <= index < len(self._assign.between(dest_buffer_id, src_buffer_id))
        return self._find(item, dict(fields, dest_buffer_id=dest_buffer_id,
                                     src_buffer_id=src_buffer_id)) is not None

    def index_of_assign_address_item(self, item=None, dest_buffer_id=None, src_buffer_id=None,
                                      **fields):
        it = self._find(item, dict(fields, dest_buffer_id=dest_buffer_id,
                                   src_buffer_id=src_buffer_id))
        if it is None:
            return None
        return self._assign.between(int(it.dest_buffer_id), int(it.src_buffer_id)).index(it)

    def ptr_assign_address_item(self, item=None, dest_buffer_id=None, src_buffer_id=None,
                                index=None, **fields):
        if item is None and index is not None:
            items = self._assign.between(dest_buffer_id, src_buffer_id)
            return items[index] if 0 <= index < len(items) else None
        return self._find(item, dict(fields, dest_buffer_id=dest_buffer_id,
                                     src_buffer_id=src_buffer_id))

    def has_assign_items(self, dest_buffer_id, src_buffer_id):
        return bool(self._assign.between(dest_buffer_id, src_buffer_id))

    def num_assign_items(self, dest_buffer_id, src_buffer_id):
        return len(self._assign.between(dest_buffer_id, src_buffer_id))

    @property
    def total_num_assign_items(self):
        return len(self._assign.items)

    def commit_address_assignments(self):
        """Check that every item names existing buffers and objects."""
        handles, cbuffers = self._buffers()
        sources = dict(cbuffers)
        sources[ARCH_PARTICLES_BUFFER_ID] = self._particles_buffer
        for it in self._assign.items:
            src, dst = sources.get(it.src_buffer_id), cbuffers.get(it.dest_buffer_id)
            if (src is None or dst is None or
                    not 0 <= it.src_elem_index < len(src.objects) or
                    not 0 <= it.dest_elem_index < len(dst.objects)):
                self._last_status = -1
                raise RuntimeError("Unable to commit address assignment items")
        self._last_status = 0
        return self

    def _perform(self, dest_buffer_id=None, src_buffer_id=None):
        handles, cbuffers = self._buffers()
        try:
            written = self._assign.perform(handles, cbuffers, dest_buffer_id, src_buffer_id)
        except (RuntimeError, IndexError) as exc:
            self._last_status = -1
            raise RuntimeError("Unable to perform assignment of address items: " + str(exc))
        self._assigned = True
        self._last_status = 0
        for bid in written:
            if bid == ARCH_BEAM_ELEMENTS_BUFFER_ID:
                self.push_beam_elements()
            else:
                handles[bid].refresh(cbuffers[bid])
        return self

    def assign_all_addresses(self):
        """Carry out every item and send what changed to the engine."""
        return self._perform()

    def assign_addresses(self, dest_buffer_id, src_buffer_id):
        if dest_buffer_id is None and src_buffer_id is None:
            return self._perform()
        if dest_buffer_id is None or src_buffer_id is None:
            raise ValueError("inconsistent dest_buffer_id and src_buffer_id parameters")
        return self._perform(dest_buffer_id, src_buffer_id)

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


class st_ParticlesAddr(C.Structure):
    """st_ParticlesAddr (particles/particles_addr.h:27-55) with the field
    names of the reference's ctypes binding (stcommon.py:517-542)."""

    _pack_ = 8
    _fields_ = [("num_particles", C.c_int64)] + [
        (name, C.c_uint64) for name in (
            "q0", "mass0", "beta0", "gamma0", "p0c", "s", "x", "y", "px", "py", "zeta",
            "psigma", "delta", "rpp", "rvv", "chi", "charge_ratio", "particle_id",
            "at_element", "at_turn", "state")]


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
    """cuda/track_job.h:42-66 / python/sixtracklib/cuda.py:565-710: a TrackJob
    bound to a CUDA node id ("platform.device"); arguments in the
    reference's order (the third is the particle set's index)."""

    def __init__(self, beam_elements_buffer, particles_buffer, particle_set_index=0,
                 until_turn_elem_by_elem=0, output_buffer=None, node_id_str=None,
                 config_str=None, **kw):
        kw.setdefault("particle_set_indices", [int(particle_set_index)])
        super().__init__(beam_elements_buffer, particles_buffer, until_turn_elem_by_elem,
                         arch="cuda", device=node_id_str, output_buffer=output_buffer,
                         config_str=config_str, **kw)

    @property
    def default_threads_per_block(self):
        return int(self._lib.st_CudaTrackJob_default_threads_per_block(self.ptr_st_track_job))

    @property
    def default_track_threads_per_block(self):
        return int(self._lib.st_CudaTrackJob_default_track_threads_per_block(
            self.ptr_st_track_job))

    # The reference's CUDA job keeps device-side arguments for the particles,
    # the beam elements and the particle addresses and a controller for its
    # node; this job holds the same data on its device.
    has_controller = property(lambda self: self.ptr_st_track_job is not None)
    has_particles_arg = property(lambda self: self.ptr_st_track_job is not None)
    has_beam_elements_arg = property(lambda self: self.ptr_st_track_job is not None)
    has_particles_addr_arg = property(lambda self: self.ptr_st_track_job is not None)
