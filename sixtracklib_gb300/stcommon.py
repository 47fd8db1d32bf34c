"""Names of the reference's ``sixtracklib.stcommon`` module that user code
imports for this path (python/sixtracklib/stcommon.py).

* The q-Gaussian helpers of ``internal/math_qgauss.h:100-190`` (used to set
  up SCQGaussProfile kicks): ``Math_q_gauss_cq``,
  ``Math_sqrt_beta_from_gauss_sigma``, ``Math_q_gauss_exp_q``,
  ``Math_q_gauss`` (optionally shifted by ``mu``) and the support limits,
  computed here in Python with the reference's formulas.
* The architecture buffer ids and status values as ctypes values (``.value``
  gives the number), and null handles (``st_NullBuffer``: None, which is
  what a failed C call returns through ctypes here).
* The string helpers (``string_to_encoded_ctypes_str``,
  ``ctypes_str_to_decoded_string``) and the ``st_TrackJobDestSrcBufferIds``
  pair (stcommon.py:29-60, 1283-1292).
* The CBuffer helpers over the C ABI (stcommon.py:320-325, 554-555,
  1196-1276).  A :class:`~sixtracklib_gb300.cbuffer.CBuffer` here keeps its
  objects in Python, not in one flat block of memory, so a "mapped" C
  buffer is a C-side copy of its image: ``st_Buffer_new_mapped_on_cbuffer``
  returns that copy (delete it with ``st_Buffer_delete``), and
  ``st_OutputBuffer_create_output_cbuffer`` writes what the C call changed
  (the monitors' particle-id ranges) back into the Python buffers.
* Every ``st_*`` function of the engine's C ABI that the package binds with
  a signature (:mod:`sixtracklib_gb300._native`), resolved on first use.
"""

from __future__ import annotations

import ctypes as ct
from math import sqrt

import numpy as np

from . import buffer as _buffer
from .cbuffer import CBuffer
from .beam_elements import q_gauss_cq as _q_gauss_cq
from .trackjob import st_ParticlesAddr  # noqa: F401  (stcommon.py:517-542)

SIXTRL_MATH_QGAUSSIAN_Q_EPS = 1e-6

st_ARCH_STATUS_SUCCESS = ct.c_int32(0)
st_ARCH_STATUS_GENERAL_FAILURE = ct.c_int32(-1)
st_TRACK_SUCCESS = ct.c_int32(0)
st_ARCH_ILLEGAL_BUFFER_ID = ct.c_uint64(_buffer.ARCH_ILLEGAL_BUFFER_ID)
st_ARCH_PARTICLES_BUFFER_ID = ct.c_uint64(_buffer.ARCH_PARTICLES_BUFFER_ID)
st_ARCH_BEAM_ELEMENTS_BUFFER_ID = ct.c_uint64(_buffer.ARCH_BEAM_ELEMENTS_BUFFER_ID)
st_ARCH_OUTPUT_BUFFER_ID = ct.c_uint64(_buffer.ARCH_OUTPUT_BUFFER_ID)
st_ARCH_ELEM_BY_ELEM_CONFIG_BUFFER_ID = ct.c_uint64(_buffer.ARCH_ELEM_BY_ELEM_CONFIG_BUFFER_ID)
st_ARCH_PARTICLE_ADDR_BUFFER_ID = ct.c_uint64(_buffer.ARCH_PARTICLE_ADDR_BUFFER_ID)
st_ARCH_MIN_USER_DEFINED_BUFFER_ID = ct.c_uint64(_buffer.ARCH_MIN_USER_DEFINED_BUFFER_ID)
st_ARCH_EXTERNAL_BUFFER_ID = ct.c_uint64(_buffer.ARCH_EXTERNAL_BUFFER_ID)
st_ARCH_MAX_USER_DEFINED_BUFFER_ID = ct.c_uint64(_buffer.ARCH_MAX_USER_DEFINED_BUFFER_ID)

st_NullBuffer = None
st_NullParticles = None
st_NullTrackJob = None
st_NullAssignAddressItem = None


# -------------------------------------------------- q-Gaussian (math_qgauss.h)
def Math_q_gauss_cq(q):
    """Normalisation c_q of the q-Gaussian (q < 3)."""
    assert q < 3.0
    return _q_gauss_cq(q)


def Math_sqrt_beta_from_gauss_sigma(sigma):
    """sqrt(beta) of the Gaussian (q = 1) of rms ``sigma``: 1 / (sqrt(2) sigma)."""
    assert sigma > 0
    return 1.0 / (sqrt(2.0) * sigma)


def Math_q_gauss_exp_q(x, q):
    """The q-exponential [1 + (1 - q) x]_+^(1 / (1 - q)), exp(x) for q = 1."""
    assert q < 3.0
    one_minus_q = 1.0 - q
    if abs(one_minus_q) >= SIXTRL_MATH_QGAUSSIAN_Q_EPS:
        u = max(1.0 + one_minus_q * x, 0.0)
        return u ** (1.0 / one_minus_q)
    return float(np.exp(x))


def Math_q_gauss(x, q, sqrt_beta, mu=None):
    """The normalised q-Gaussian at ``x`` (centred at ``mu`` if given)."""
    assert q < 3.0 and sqrt_beta > 0.0
    if mu is not None:
        x = x - mu
    cq = Math_q_gauss_cq(q)
    return (sqrt_beta / cq) * Math_q_gauss_exp_q(-(sqrt_beta * sqrt_beta * x * x), q)


def Math_q_gauss_min_support(q, sqrt_beta):
    """Lower end of the support: -1 / sqrt(beta (1 - q)) for q < 1, else -1e10."""
    assert q < 3.0 and sqrt_beta > 0.0
    return -1e10 if q >= 1.0 else -1.0 / sqrt(sqrt_beta * sqrt_beta * (1.0 - q))


def Math_q_gauss_max_support(q, sqrt_beta):
    """Upper end of the support: 1 / sqrt(beta (1 - q)) for q < 1, else 1e10."""
    assert q < 3.0 and sqrt_beta > 0.0
    return 1e10 if q >= 1.0 else 1.0 / sqrt(sqrt_beta * sqrt_beta * (1.0 - q))


# ------------------------------------------------------------ strings
def string_to_encoded_ctypes_str(s, encoding="utf-8", strip=True):
    """``s`` as a NUL-terminated ctypes char buffer (None stays None)."""
    if s is None:
        return None
    if strip:
        s = s.strip()
    return ct.create_string_buffer(s.encode(encoding))


def ctypes_str_to_decoded_string(bstr, encoding="utf-8", strip=True):
    """A ctypes char buffer, ``bytes`` or ``c_char_p`` value as a str."""
    if bstr is None:
        return None
    raw = bstr.value if hasattr(bstr, "value") else bstr
    if raw is None:
        return None
    out = raw.decode(encoding) if isinstance(raw, (bytes, bytearray)) else str(raw)
    out = out.split("\0", 1)[0]
    return out.strip() if strip else out


class st_TrackJobDestSrcBufferIds(ct.Structure):
    """A (destination, source) buffer-id pair of an address assignment."""

    _pack_ = 8
    _fields_ = [("dest_buffer_id", ct.c_uint64), ("src_buffer_id", ct.c_uint64)]


st_TrackJobDestSrcBufferIds_p = ct.POINTER(st_TrackJobDestSrcBufferIds)
st_NullTrackJobDestSrcBufferIds = ct.cast(0, st_TrackJobDestSrcBufferIds_p)


# ------------------------------------------------------------ CBuffers
def _lib():
    from . import _native

    return _native.load()


def st_Buffer_new_mapped_on_cbuffer(cbuffer):
    """A C st_Buffer with a copy of ``cbuffer``'s image (remapped to its own
    address); the caller deletes it with ``st_Buffer_delete``."""
    img = _buffer.get_cbuffer_from_obj(cbuffer).to_image()
    return _lib().st_Buffer_new_on_data(img.ctypes.data, img.nbytes)


def st_Particles_cbuffer_get_particles(cbuffer, obj_index):
    """An ``st_Particles*`` for object ``obj_index`` of ``cbuffer``: it
    points into a C-side copy of the buffer that lives as long as
    ``cbuffer`` and shows its contents as of this call; None if the object
    is not a particle set."""
    cb = _buffer.get_cbuffer_from_obj(cbuffer)
    handle = _buffer.CBufferHandle(cb)
    views = cb.__dict__.setdefault("_st_particle_views", [])
    views.append(handle)
    return _lib().st_Particles_buffer_get_particles(handle.ptr, int(obj_index)) or None


def st_OutputBuffer_create_output_cbuffer(beam_elements_buffer, particles_buffer,
                                          num_particle_sets=1, indices=None,
                                          until_turn_elem_by_elem=0):
    """The output buffer a tracking run of ``particles_buffer`` through
    ``beam_elements_buffer`` writes: (CBuffer, elem-by-elem output offset,
    beam-monitor output offset, first turn), or (None, -1, -1, -1) when
    nothing is to be stored or the inputs are invalid.  Built by
    st_OutputBuffer_calculate_output_buffer_params and st_OutputBuffer_prepare;
    the monitors' particle-id ranges set by the latter are written back into
    ``beam_elements_buffer``.  Particle sets: ``indices`` (default: the first
    ``num_particle_sets`` objects)."""
    L = _lib()
    pcb = _buffer.get_cbuffer_from_obj(particles_buffer)
    ecb = _buffer.get_cbuffer_from_obj(beam_elements_buffer)
    ph, eh = _buffer.CBufferHandle(pcb), _buffer.CBufferHandle(ecb)
    out = None
    try:
        n = int(num_particle_sets)
        idx = list(indices) if indices is not None else list(range(n))
        arr = (ct.c_uint64 * max(len(idx), 1))(*idx)
        until = int(until_turn_elem_by_elem)
        sizes = [ct.c_uint64(0) for _ in range(4)]
        rc = L.st_OutputBuffer_calculate_output_buffer_params_for_particles_sets(
            eh.ptr, ph.ptr, len(idx), arr, until, *[ct.byref(x) for x in sizes], 8)
        if rc != 0 or sizes[0].value == 0:
            return None, -1, -1, -1
        out = L.st_Buffer_new_detailed(sizes[0].value, sizes[1].value, sizes[2].value,
                                       sizes[3].value, 0)
        ebe, mon, turn = ct.c_uint64(0), ct.c_uint64(0), ct.c_int64(0)
        rc = L.st_OutputBuffer_prepare_for_particle_sets(
            eh.ptr, out, ph.ptr, len(idx), arr, until, ct.byref(ebe), ct.byref(mon),
            ct.byref(turn))
        if rc != 0:
            return None, -1, -1, -1
        eh.pull_into(ecb)
        size = L.st_Buffer_get_size(out)
        data = ct.cast(L.st_Buffer_get_const_data_begin(out), ct.POINTER(ct.c_uint64))
        img = np.ctypeslib.as_array(data, shape=(size // 8,)).copy()
        return CBuffer.from_image(img), ebe.value, mon.value, turn.value
    finally:
        if out:
            L.st_Buffer_delete(out)
        ph.free()
        eh.free()


# ------------------------------------------------------------ C functions
def __getattr__(name):
    if name.startswith("st_"):
        from . import _native

        if name in _native._SIGNATURES:
            return getattr(_native.load(), name)
        raise AttributeError(f"{name} is not part of this engine's bound C ABI "
                             f"(see include/sixtracklib_gb300.h and _native)")
    raise AttributeError(name)
