"""Host-side entry points of the C ABI on the CPU: every beam-element
constructor (NS(X_new), NS(X_add)), the buffer's object access, the
particle-set helpers and the elem-by-elem configuration, each checked
against the Python encoder, the particle formulas or the oracle.  Nothing
here needs a GPU."""

import ctypes as C

import numpy as np
import pytest

from oracle.pyoracle import EbeConfig, Oracle
from sixtracklib_gb300 import CBuffer, _native
from sixtracklib_gb300.beam_elements import Elements
from tests import capi

D, I64, U64, VP, B = C.c_double, C.c_int64, C.c_uint64, C.c_void_p, C.c_bool


@pytest.fixture(scope="module")
def lib():
    _native.load()
    L = C.CDLL(_native.lib_path())  # own prototypes, not the shared handle's
    for name, args, res in (("st_Buffer_new", [U64], VP), ("st_Buffer_delete", [VP], None),
                            ("st_Buffer_get_size", [VP], U64),
                            ("st_Buffer_get_const_data_begin", [VP], VP),
                            ("st_Buffer_get_num_of_objects", [VP], U64),
                            ("st_Buffer_get_const_object", [VP, U64], VP),
                            ("st_Particles_new", [VP, U64], VP)):
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res
    sigs = {
        "st_Drift_new": [VP], "st_Drift_add": [VP, D],
        "st_DriftExact_new": [VP], "st_DriftExact_add": [VP, D],
        "st_Multipole_new": [VP, I64], "st_Multipole_add": [VP, I64, VP, D, D, D],
        "st_Multipole_bal": [VP],
        "st_RFMultipole_new": [VP, I64], "st_RFMultipole_add": [VP, I64, D, D, D, VP, VP],
        "st_Cavity_new": [VP], "st_Cavity_add": [VP, D, D, D],
        "st_XYShift_new": [VP], "st_XYShift_add": [VP, D, D],
        "st_SRotation_new": [VP], "st_SRotation_add": [VP, D],
        "st_SRotation_add_detailed": [VP, D, D],
        "st_LimitRect_new": [VP], "st_LimitRect_add": [VP, D, D, D, D],
        "st_LimitEllipse_new": [VP], "st_LimitEllipse_add": [VP, D, D],
        "st_LimitRectEllipse_new": [VP], "st_LimitRectEllipse_add": [VP, D, D, D, D],
        "st_DipoleEdge_new": [VP], "st_DipoleEdge_add": [VP, D, D],
        "st_BeamMonitor_new": [VP], "st_BeamMonitor_add": [VP, I64, I64, I64, U64, I64, I64, B, B],
        "st_BeamBeam4D_new": [VP, U64], "st_BeamBeam4D_add": [VP, U64, VP],
        "st_BeamBeam6D_new": [VP, U64], "st_BeamBeam6D_add": [VP, U64, VP],
        "st_SCCoasting_new": [VP], "st_SCCoasting_add": [VP, D, D, D, D, D, D, D, D, B],
        "st_SCQGaussProfile_new": [VP],
        "st_SCQGaussProfile_add": [VP, D, D, D, D, D, D, D, D, D, B],
        "st_Buffer_get_objects_begin": [VP], "st_Buffer_get_objects_end": [VP],
        "st_Buffer_get_const_objects_begin": [VP], "st_Buffer_get_const_objects_end": [VP],
        "st_Buffer_get_object": [VP, U64], "st_Buffer_get_data_begin": [VP],
        "st_Buffer_add_object": [VP, VP, U64, U64, U64, VP, VP, VP],
        "st_Particles_add_copy": [VP, VP], "st_Particles_buffer_get_const_particles": [VP, U64],
        "st_Particles_set_reference": [VP, D, D, D],
        "st_Particles_update_delta_value": [VP, I64, D],
    }
    for name, args in sigs.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = VP
    for name in ("st_Particles_set_reference", "st_Particles_update_delta_value"):
        getattr(L, name).restype = None
    for name, args, res in (
            ("st_Object_get_type_id", [VP], U64), ("st_Object_get_begin_addr", [VP], U64),
            ("st_Object_get_size", [VP], U64), ("st_Particles_get_num_of_particles", [VP], I64),
            ("st_Particles_buffer_get_num_of_particle_blocks", [VP], U64),
            ("st_Particles_copy", [VP, VP], C.c_int32),
            ("st_ElemByElemConfig_init_detailed", [VP, I64, I64, I64, I64, I64, I64, I64, B],
             C.c_int32),
            ("st_ElemByElemConfig_get_particles_store_index_details", [VP, I64, I64, I64], I64),
            ("st_ElemByElemConfig_get_stored_num_particles", [VP], I64)):
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res
    return L


def _image(ptr, L):
    n = L.st_Buffer_get_size(ptr)
    data = L.st_Buffer_get_const_data_begin(ptr)
    return np.ctypeslib.as_array(C.cast(data, C.POINTER(C.c_uint64)), shape=(n // 8,)).copy()


def _objects(cb):
    return [(o.typeid, o.words.tobytes(), tuple(o.ptr_fields)) for o in cb.objects]


def _dbl(*v):
    return (C.c_double * len(v))(*v)


def test_element_add_constructors_match_the_python_encoder(lib):
    """NS(X_add) for every beam element the reference's C API has: the same
    objects, byte for byte, as the Python classes with the same parameters."""
    L = lib
    b = L.st_Buffer_new(0)
    try:
        assert L.st_Drift_add(b, 1.5)
        assert L.st_DriftExact_add(b, 0.7)
        assert L.st_Multipole_add(b, 2, _dbl(1e-4, 2e-4, 0.05, 0.0, 0.3, 0.1), 1.0, 1e-5, -2e-5)
        assert L.st_RFMultipole_add(b, 1, 1e5, 4e8, 30.0, _dbl(1e-6, 0.0, 0.002, 1e-4),
                                    _dbl(10.0, 5.0, 20.0, 6.0))
        assert L.st_Cavity_add(b, 6e6, 4e8, 180.0)
        assert L.st_XYShift_add(b, 1e-4, -2e-4)
        assert L.st_SRotation_add_detailed(b, np.cos(0.01), np.sin(0.01))
        assert L.st_LimitRect_add(b, -0.02, 0.03, -0.01, 0.04)
        assert L.st_LimitEllipse_add(b, 0.015, 0.01)
        assert L.st_LimitRectEllipse_add(b, 0.03, 0.02, 0.035 ** 2, 0.025 ** 2)
        assert L.st_DipoleEdge_add(b, 0.01, -0.02)
        # min_particle_id before max_particle_id, as be_monitor.h:419-425
        assert L.st_BeamMonitor_add(b, 4, 1, 2, 0, 0, 63, True, False)
        bb4 = _dbl(*np.arange(1.0, 12.0))
        assert L.st_BeamBeam4D_add(b, 11, bb4)
        bb6 = _dbl(*np.linspace(0.5, 3.0, 47))
        assert L.st_BeamBeam6D_add(b, 47, bb6)
        assert L.st_SCCoasting_add(b, 1e11, 1000.0, 1e-3, 1.5e-3, 1.0, 1e-5, -1e-5, 1e-10, True)
        assert L.st_SCQGaussProfile_add(b, 1e11, 0.1, 1e-3, 1.2e-3, 1.0, 0.0, 0.0, 1e-10, 1.0,
                                        True)
        cb = CBuffer.from_image(_image(b, L))
    finally:
        L.st_Buffer_delete(b)
    e = Elements()
    e.Drift(length=1.5)
    e.DriftExact(length=0.7)
    m = e.Multipole(knl=[1e-4, 0.05, 0.6], ksl=[2e-4, 0.0, 0.2], length=1.0, hxl=1e-5,
                    hyl=-2e-5)
    e.RFMultipole(voltage=1e5, frequency=4e8, lag=30.0, knl=[1e-6, 0.002], ksl=[0.0, 1e-4],
                  pn=[10.0, 20.0], ps=[5.0, 6.0])
    e.Cavity(voltage=6e6, frequency=4e8, lag=180.0)
    e.XYShift(dx=1e-4, dy=-2e-4)
    e.SRotation(cos_z=np.cos(0.01), sin_z=np.sin(0.01))
    e.LimitRect(min_x=-0.02, max_x=0.03, min_y=-0.01, max_y=0.04)
    e.LimitEllipse(a=0.015, b=0.01)
    e.LimitRectEllipse(max_x=0.03, max_y=0.02, a=0.035, b=0.025)
    e.DipoleEdge(r21=0.01, r43=-0.02)
    e.BeamMonitor(num_stores=4, start=1, skip=2, out_address=0, max_particle_id=63,
                  min_particle_id=0, is_rolling=1, is_turn_ordered=0)
    e.BeamBeam4D(data=np.arange(1.0, 12.0))
    e.BeamBeam6D(data=np.linspace(0.5, 3.0, 47))
    e.SCCoasting(number_of_particles=1e11, circumference=1000.0, sigma_x=1e-3, sigma_y=1.5e-3,
                 length=1.0, x_co=1e-5, y_co=-1e-5, min_sigma_diff=1e-10, enabled=1)
    e.SCQGaussProfile(number_of_particles=1e11, bunchlength_rms=0.1, sigma_x=1e-3,
                      sigma_y=1.2e-3, length=1.0, min_sigma_diff=1e-10, q_param=1.0, enabled=1)
    assert np.allclose(m.bal, [1e-4, 2e-4, 0.05, 0.0, 0.3, 0.1], rtol=1e-15, atol=0)
    assert _objects(cb) == _objects(e.cbuffer)


def test_element_new_constructors_and_bal_access(lib):
    """NS(X_new) appends an object of the element's type and struct size
    (the size NS(X_add) gives); NS(Multipole_new) reserves 2 (order + 1)
    coefficients, which st_Multipole_bal writes in place."""
    L = lib
    news = [("st_Drift_new", ()), ("st_DriftExact_new", ()), ("st_Cavity_new", ()),
            ("st_XYShift_new", ()), ("st_SRotation_new", ()), ("st_LimitRect_new", ()),
            ("st_LimitEllipse_new", ()), ("st_LimitRectEllipse_new", ()),
            ("st_DipoleEdge_new", ()), ("st_BeamMonitor_new", ()), ("st_SCCoasting_new", ()),
            ("st_SCQGaussProfile_new", ()), ("st_Multipole_new", (3,)),
            ("st_RFMultipole_new", (2,)), ("st_BeamBeam4D_new", (11,)),
            ("st_BeamBeam6D_new", (47,))]
    b = L.st_Buffer_new(0)
    try:
        for name, args in news:
            assert getattr(L, name)(b, *args), name
        mp = L.st_Buffer_get_object(b, 12)
        begin = C.cast(mp, C.POINTER(C.c_uint64))[0]
        bal = L.st_Multipole_bal(begin)
        vals = [0.0, 0.0, 0.05, 0.0, 0.3, 0.0, 0.001, 0.0]  # bal[2k] = knl[k] / k!
        for k, v in enumerate(vals):
            C.cast(bal, C.POINTER(C.c_double))[k] = v
        cb = CBuffer.from_image(_image(b, L))
    finally:
        L.st_Buffer_delete(b)
    e = Elements()
    e.Drift(length=0.0)
    e.DriftExact(length=0.0)
    e.Cavity(voltage=0.0, frequency=0.0, lag=0.0)
    e.XYShift(dx=0.0, dy=0.0)
    e.SRotation(cos_z=1.0, sin_z=0.0)
    e.LimitRect()
    e.LimitEllipse()
    e.LimitRectEllipse()
    e.DipoleEdge(r21=0.0, r43=0.0)
    e.BeamMonitor()
    e.SCCoasting()
    e.SCQGaussProfile()
    e.Multipole(knl=[0.0, 0.05, 0.6, 0.006])
    e.RFMultipole(knl=[0.0, 0.0, 0.0], ksl=[0.0, 0.0, 0.0], pn=[0.0, 0.0, 0.0],
                  ps=[0.0, 0.0, 0.0])
    e.BeamBeam4D(data=np.zeros(11))
    e.BeamBeam6D(data=np.zeros(47))
    assert [o.typeid for o in cb.objects] == [o.typeid for o in e.cbuffer.objects]
    assert [o.words.size for o in cb.objects] == [o.words.size for o in e.cbuffer.objects]
    mp_c, mp_py = cb.objects[12], e.cbuffer.objects[12]
    assert mp_c.words.tobytes() == mp_py.words.tobytes()


def test_buffer_object_access(lib):
    """NS(Buffer_get_objects_begin / _end / get_object) and the NS(Object)
    accessors agree with the image: 24-byte index entries {begin address,
    type id, size} in element order, the const and non-const forms alike;
    NS(Buffer_add_object) appends a generic object with its arrays."""
    L = lib
    e = Elements()
    e.Drift(length=2.0)
    e.Multipole(knl=[0.0, 0.05])
    e.Cavity(voltage=1.0, frequency=2.0, lag=3.0)
    img = e.cbuffer.to_image()
    b = capi.c_buffer_from_image(img)
    try:
        n = L.st_Buffer_get_num_of_objects(b)
        assert n == 3
        begin, end = L.st_Buffer_get_objects_begin(b), L.st_Buffer_get_objects_end(b)
        assert end - begin == 24 * n
        assert L.st_Buffer_get_const_objects_begin(b) == begin
        assert L.st_Buffer_get_const_objects_end(b) == end
        assert L.st_Buffer_get_data_begin(b) == L.st_Buffer_get_const_data_begin(b)
        for i, o in enumerate(e.cbuffer.objects):
            obj = L.st_Buffer_get_object(b, i)
            assert obj == begin + 24 * i
            assert L.st_Object_get_type_id(obj) == o.typeid
            addr = L.st_Object_get_begin_addr(obj)
            assert L.st_Object_get_size(obj) >= 8 * o.words.size
            first = C.cast(addr, C.POINTER(C.c_uint64))[0]
            assert first == int(o.words[0])
        # generic append: a Drift struct, then a multipole with its bal array
        length = C.c_double(4.5)
        assert L.st_Buffer_add_object(b, C.addressof(length), 8, 2, 0, None, None, None)
        mp = (C.c_uint64 * 5)(1, np.float64(0.0).view(np.uint64), 0, 0, 0)
        bal = _dbl(0.0, 0.0, -0.05, 0.0)
        field = (C.c_uint64 * 1)(4)
        arrays = (C.c_void_p * 1)(C.cast(bal, C.c_void_p))
        words = (C.c_uint64 * 1)(4)
        assert L.st_Buffer_add_object(b, mp, 40, 4, 1, field, arrays, words)
        cb = CBuffer.from_image(_image(b, L))
    finally:
        L.st_Buffer_delete(b)
    e.Drift(length=4.5)
    e.Multipole(knl=[0.0, -0.05])
    assert _objects(cb) == _objects(e.cbuffer)


def test_particle_set_helpers(lib):
    """NS(Particles_new / _add_copy / _copy / _get_num_of_particles), the
    const getter and the block count; NS(Particles_set_reference) and
    NS(Particles_update_delta_value) give the reference quantities and the
    delta-dependent columns the oracle's formulas give
    (particles.h:5459-5496)."""
    L = lib
    b = L.st_Buffer_new(0)
    try:
        p = L.st_Particles_new(b, 5)
        assert p and L.st_Particles_get_num_of_particles(p) == 5
        L.st_Particles_set_reference(p, 7e12, 938272088.16, 1.0)
        for i, d in enumerate([0.0, 1e-4, -3e-4, 2e-3, -1e-5]):
            L.st_Particles_update_delta_value(p, i, d)
        q = L.st_Particles_add_copy(b, p)
        assert q and L.st_Buffer_get_num_of_objects(b) == 2
        assert L.st_Particles_buffer_get_num_of_particle_blocks(b) == 2
        assert L.st_Particles_buffer_get_const_particles(b, 1) == q
        r = L.st_Particles_new(b, 5)
        assert L.st_Particles_copy(r, p) == 0
        cb = CBuffer.from_image(_image(b, L))
    finally:
        L.st_Buffer_delete(b)
    from sixtracklib_gb300.particles import Particles

    parts = [Particles._from_cobject(o, cb, i) for i, o in enumerate(cb.objects)]
    a, c, d = (x.block for x in parts)
    assert np.array_equal(a, c) and np.array_equal(a, d)
    f = a[:17].view(np.float64)
    mass0, p0c = 938272088.16, 7e12
    energy0 = np.sqrt(p0c * p0c + mass0 * mass0)
    assert np.allclose(f[3], energy0 / mass0, rtol=1e-15)             # gamma0
    assert np.allclose(f[2], p0c / energy0, rtol=1e-15)               # beta0
    delta = np.array([0.0, 1e-4, -3e-4, 2e-3, -1e-5])
    assert np.array_equal(f[12], delta)
    assert np.allclose(f[13], 1.0 / (1.0 + delta), rtol=1e-15)        # rpp
    beta0 = f[2]
    ptau_beta0 = np.sqrt((delta * beta0) ** 2 + 2 * delta * beta0 * beta0 + 1) - 1
    assert np.allclose(f[14], (1 + delta) / (1 + ptau_beta0), rtol=1e-15)  # rvv
    assert np.allclose(f[11], ptau_beta0 / (beta0 * beta0), rtol=1e-12, atol=1e-20)


def test_elem_by_elem_config_matches_the_oracle(lib):
    """NS(ElemByElemConfig_init_detailed), the store index of a particle at an
    element and turn, and the stored particle count, against the oracle's
    restatement of output/elem_by_elem_config.h:667-763, rolling and not,
    indices inside and outside the configured ranges; the reference's one
    order (ELEM_BY_ELEM_ORDER_TURN_ELEM_PARTICLES = 0) only, and empty or
    negative ranges rejected."""
    L = lib
    orc = Oracle()
    bad = capi.StElemByElemConfig()
    for args in ((1, 2, 9, 1, 6, 0, 3), (0, 9, 2, 1, 6, 0, 3), (0, 2, 9, 6, 1, 0, 3),
                 (0, -1, 9, 1, 6, 0, 3), (0, 2, 9, 1, 6, 3, 0)):
        assert L.st_ElemByElemConfig_init_detailed(C.byref(bad), *args, False) == -1, args
    for order, rolling in ((0, False), (0, True)):
        cfg = capi.StElemByElemConfig()
        assert L.st_ElemByElemConfig_init_detailed(C.byref(cfg), order, 2, 9, 1, 6, 0, 3,
                                                   rolling) == 0
        n = L.st_ElemByElemConfig_get_stored_num_particles(C.byref(cfg))
        assert n == (9 - 2 + 1) * (6 - 1 + 1) * (3 - 0 + 1)
        ocfg = EbeConfig(*[getattr(cfg, name) for name, _ in EbeConfig._fields_])
        for pid in range(0, 12):
            for elem in range(0, 9):
                for turn in range(-1, 7):
                    got = L.st_ElemByElemConfig_get_particles_store_index_details(
                        C.byref(cfg), pid, elem, turn)
                    assert got == orc.ebe_store_index(ocfg, pid, elem, turn), \
                        (order, rolling, pid, elem, turn)


def test_jobs_and_single_particle_calls_fail_loudly_without_a_gpu(lib):
    """No CPU fallback for jobs either: every TrackJob / TrackJobNew /
    CudaTrackJob constructor returns NULL on a machine without a GPU and
    names the reason; the reference's other architectures are refused by
    name; the single-particle tracking calls fail and leave the particle as
    it was; the CUDA node list is empty."""
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    L = lib
    e = Elements()
    e.Drift(length=1.0)
    img = e.cbuffer.to_image()
    from sixtracklib_gb300 import ParticlesSet, lattices

    ps = ParticlesSet()
    ps.Particles(num_particles=2).set_block(lattices.gaussian_particles(2).block)
    pimg = ps.cbuffer.to_image()
    eb = capi.c_buffer_from_image(img)
    pb = capi.c_buffer_from_image(pimg)
    cs = C.c_char_p
    try:
        calls = [
            ("st_TrackJob_create", [cs, cs], (b"cuda", b"")),
            ("st_TrackJob_new", [cs, VP, VP, cs], (b"cuda", pb, eb, b"")),
            ("st_TrackJob_new_with_output", [cs, VP, VP, VP, U64, cs], (b"cuda", pb, eb, None, 0, b"")),
            ("st_TrackJobNew_create", [cs, cs], (b"cuda", b"")),
            ("st_CudaTrackJob_create", [], ()),
            ("st_CudaTrackJob_new_from_config_str", [cs], (b"mode=fast",)),
            ("st_CudaTrackJob_new", [cs, VP, VP], (b"0.0", pb, eb)),
            ("st_CudaTrackJob_new_with_output", [cs, VP, VP, VP, U64], (b"0.0", pb, eb, None, 0)),
            ("st_CudaTrackJob_new_detailed", [cs, VP, U64, VP, VP, VP, U64, cs],
             (b"0.0", pb, 0, None, eb, None, 0, b"")),
        ]
        for name, args, vals in calls:
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = VP
            assert not fn(*vals), name
            err = _native.last_error()
            assert "GPU" in err or "CUDA" in err or "device" in err, (name, err)
        L.st_TrackJob_create.argtypes = [cs, cs]
        L.st_TrackJob_create.restype = VP
        for arch in (b"cpu", b"opencl"):
            assert not L.st_TrackJob_create(arch, b"")
            assert "architecture" in _native.last_error()
        fn = L.st_CudaTrackJob_get_available_node_indices_list
        fn.argtypes = [U64, VP]
        fn.restype = U64
        out = (C.c_int64 * 4)(-7, -7, -7, -7)
        assert fn(4, out) == 0 and list(out) == [-7] * 4
        # single-particle free functions (track.h:86-132)
        q = lattices.gaussian_particles(3)
        blk = q.block.copy()
        sp = capi.particles_view(blk)
        L.st_Track_particle_line.argtypes = [VP, I64, VP, U64, U64, C.c_bool]
        L.st_Track_particle_line.restype = C.c_int32
        assert L.st_Track_particle_line(C.byref(sp), 1, eb, 0, 1, True) == -1
        cfg = capi.StElemByElemConfig()
        assert L.st_ElemByElemConfig_init_detailed(C.byref(cfg), 0, 0, 2, 0, 0, 0, 0, False) == 0
        fn = L.st_Track_particle_element_by_element_until_turn
        fn.argtypes = [VP, I64, VP, VP, I64]
        fn.restype = C.c_int32
        assert fn(C.byref(sp), 1, C.byref(cfg), eb, 1) == -1
        assert np.array_equal(blk, q.block)
    finally:
        L.st_Buffer_delete(eb)
        L.st_Buffer_delete(pb)


def test_every_job_call_is_null_safe(lib):
    """A NULL job is an error, not a crash (internal/track_job.cpp:417-445):
    every TrackJob / TrackJobNew / CudaTrackJob call the header declares,
    given NULL for the job and zeros for the rest, returns -1 where it
    returns a status and 0 / false / NULL from the getters (an empty string
    for the string getters)."""
    import re

    import os

    header = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                          "include", "sixtracklib_gb300.h")
    with open(header) as f:
        hdr = f.read()
    # a handle of its own: the prototypes set below must not leak into the
    # shared one the other tests use
    lib = C.CDLL(_native.lib_path())
    decls = re.findall(r"^([A-Za-z_][A-Za-z0-9_ \*]*?)\b(st_(?:TrackJob|TrackJobNew|CudaTrackJob)"
                       r"_[A-Za-z0-9_]+)\s*\(([^;]*?)\);", hdr, re.M | re.S)
    called = 0
    for ret, name, args in decls:
        args = [a.strip() for a in " ".join(args.split()).split(",")]
        if not args or args == ["void"] or "TrackJob" not in args[0]:
            continue
        ret = " ".join(ret.split())
        fn = getattr(lib, name)
        fn.argtypes = [C.c_void_p] * len(args)
        if ret == "void":
            fn.restype = None
        elif ret in ("st_track_status_t", "int32_t"):
            fn.restype = C.c_int32
        elif ret == "const char *":
            fn.restype = C.c_char_p
        elif ret == "bool":
            fn.restype = C.c_bool
        else:
            fn.restype = C.c_uint64
        r = fn(*([None] * len(args)))
        called += 1
        if ret in ("st_track_status_t", "int32_t"):
            assert r == -1, name
        elif ret == "const char *":
            assert r == b"", name
        elif ret == "bool":
            assert r is False, name
        elif ret.endswith("*"):
            assert r in (0, None), name
    assert called > 100


def test_python_job_names_of_the_reference_over_a_null_job():
    """The Python job's TrackJobBaseNew names (debug mode, collect flags,
    output offsets, deprecated camelCase spellings; trackjob.py:150-1210)
    reach the C ABI; on a NULL job they answer as a NULL job does: status
    operations raise, getters are empty."""
    import warnings as w

    from sixtracklib_gb300 import CBuffer
    from sixtracklib_gb300.trackjob import CudaTrackJob

    job = object.__new__(CudaTrackJob)
    job._lib = _native.load()
    job.ptr_st_track_job = None
    job._pset_indices = []
    job._last_status = 0
    job._particles_buffer = CBuffer()
    job._stored = {}
    assert job.is_in_debug_mode is False and job.debug_register == 0
    for op in (job.enable_debug_mode, job.disable_debug_mode, job.collect_debug_flag,
               job.collect_particle_addresses):
        with pytest.raises(RuntimeError):
            op()
    assert job.last_status == -1
    assert job.pointer is None and job.total_num_particles == 0 and job.collecting_flags == 0
    assert not (job.is_collecting_beam_elements or job.is_collecting_output or
                job.has_config_str or job.has_elem_by_elem_config or job.has_beam_monitors)
    assert job.num_elem_by_elem_turn == 0
    assert job.elem_by_elem_output_buffer_offset == job.beam_monitor_output_buffer_offset == 0
    assert not job.uses_arguments and not job.uses_controller
    with w.catch_warnings(record=True) as caught:
        w.simplefilter("always")
        assert job.collectOutput() is job
        assert job.collectParticles() is job
        with pytest.raises(RuntimeError):
            job.collectDebugFlag()
        with pytest.raises(RuntimeError):
            job.collectParticlesAddresses()
    assert sum(issubclass(c.category, DeprecationWarning) for c in caught) == 4
    job.ptr_st_track_job = None  # __del__ has nothing to release
