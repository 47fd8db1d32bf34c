"""ctypes views of the C ABI structs used by the tests (st_Particles,
st_ElemByElemConfig, the generic-address output descriptor)."""

import ctypes as C

import numpy as np

from sixtracklib_gb300 import _native


class StParticles(C.Structure):
    _fields_ = [("num_particles", C.c_int64)] + [(f"c{i}", C.c_void_p) for i in range(21)]


class StElemByElemConfig(C.Structure):
    _fields_ = [(n, C.c_int64) for n in (
        "order", "num_particles_to_store", "num_elements_to_store", "num_turns_to_store",
        "min_particle_id", "min_element_id", "min_turn", "max_particle_id", "max_element_id",
        "max_turn", "is_rolling")] + [("out_store_addr", C.c_uint64)]


class GenericAddr(C.Structure):
    _fields_ = [("num_particles", C.c_int64)] + [(f"a{i}", C.c_uint64) for i in range(21)]


def particles_view(block: np.ndarray) -> StParticles:
    """st_Particles whose column pointers point into a 21 x n numpy block."""
    assert block.flags.c_contiguous
    n = block.shape[1]
    sp = StParticles()
    sp.num_particles = n
    for c in range(21):
        setattr(sp, f"c{c}", block.ctypes.data + c * n * 8)
    return sp


def generic_addr(block: np.ndarray) -> GenericAddr:
    n = block.shape[1]
    g = GenericAddr()
    g.num_particles = n
    for c in range(21):
        setattr(g, f"a{c}", block.ctypes.data + c * n * 8)
    return g


def c_buffer_from_image(img: np.ndarray):
    lib = _native.load()
    ptr = lib.st_Buffer_new_on_data(img.ctypes.data, img.nbytes)
    assert ptr, _native.last_error()
    return ptr


def lib():
    L = _native.load()
    vp = C.c_void_p
    L.st_Track_all_particles_element_by_element_until_turn.argtypes = [vp, vp, vp, C.c_int64]
    L.st_Track_all_particles_element_by_element_until_turn.restype = C.c_int32
    L.st_Track_particle_until_turn.argtypes = [vp, C.c_int64, vp, C.c_int64]
    L.st_Track_particle_until_turn.restype = C.c_int32
    return L
