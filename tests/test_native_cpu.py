"""The C ABI library on the CPU: it loads, exports every entry point the
header declares, and its CObjects buffer agrees byte-for-byte in content with
the Python encoder and with the reference's files.  No tracking call runs
here (tracking needs the GPU)."""

import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from sixtracklib_gb300 import CBuffer, _native, lattices
from sixtracklib_gb300.beam_elements import Elements
from tests import capi
from tests.conftest import reference_testdata


@pytest.fixture(scope="module")
def lib():
    return _native.load()


def test_library_exports_every_declared_symbol(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", _native.lib_path()],
                         capture_output=True, text=True, check=True).stdout
    syms = {line.split()[-1] for line in out.splitlines() if line.strip()}
    declared = _native.exported_symbols_expected()
    assert len(declared) > 150
    missing = [s for s in declared if s not in syms]
    assert not missing, missing


def _objects(cb):
    return [(o.typeid, o.words.tobytes(), tuple(o.ptr_fields)) for o in cb.objects]


def c_image(ptr, lib):
    n = lib.st_Buffer_get_size(ptr)
    data = lib.st_Buffer_get_const_data_begin(ptr)
    return np.ctypeslib.as_array(C.cast(data, C.POINTER(C.c_uint64)), shape=(n // 8,)).copy()


def test_python_and_c_buffers_agree(lib):
    e = lattices.bb_sc_ring()
    e.BeamMonitor(num_stores=3, start=1, skip=2)
    e.RFMultipole(voltage=1.0, frequency=2.0, lag=3.0, knl=[1, 2], ksl=[3], pn=[4], ps=[5, 6])
    img = e.cbuffer.to_image()
    ptr = capi.c_buffer_from_image(img)
    try:
        assert lib.st_Buffer_get_num_of_objects(ptr) == len(e)
        back = CBuffer.from_image(c_image(ptr, lib))
        assert _objects(back) == _objects(e.cbuffer)
    finally:
        lib.st_Buffer_delete(ptr)


def test_c_element_constructors(lib):
    L = lib
    L.st_Cavity_add.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_double]
    L.st_Cavity_add.restype = C.c_void_p
    L.st_LimitEllipse_add.argtypes = [C.c_void_p, C.c_double, C.c_double]
    L.st_LimitEllipse_add.restype = C.c_void_p
    b = L.st_Buffer_new(0)
    try:
        for k in range(300):  # forces several re-layouts of the sections
            assert L.st_Drift_add(b, 0.5 + k)
        bal = (C.c_double * 4)(0.0, 0.0, 0.05, 0.0)
        assert L.st_Multipole_add(b, 1, bal, 0.0, 0.0, 0.0)
        assert L.st_Cavity_add(b, 6e6, 4e8, 180.0)
        assert L.st_LimitEllipse_add(b, 0.015, 0.01)
        assert L.st_Particles_new(b, 10)
        cb = CBuffer.from_image(c_image(b, L))
    finally:
        L.st_Buffer_delete(b)
    ref = Elements()
    for k in range(300):
        ref.Drift(length=0.5 + k)
    ref.Multipole(knl=[0.0, 0.05])
    ref.Cavity(voltage=6e6, frequency=4e8, lag=180.0)
    ref.LimitEllipse(a=0.015, b=0.01)
    assert _objects(cb)[:-1] == _objects(ref.cbuffer)
    assert cb.objects[-1].typeid == 1 and int(cb.objects[-1].words[0]) == 10


def test_reference_files_load_identically(lib):
    for parts in (("bbsimple", "beam_elements.bin"), ("beambeam", "beam_elements.bin"),
                  ("lhc_no_bb", "beam_elements.bin"), ("bbsimple", "particles_dump.bin")):
        path = reference_testdata(*parts)
        if path is None:
            pytest.skip("reference test data not mounted")
        py = CBuffer.fromfile(path)
        ptr = lib.st_Buffer_new_from_file(path.encode())
        assert ptr, _native.last_error()
        try:
            cb = CBuffer.from_image(c_image(ptr, lib))
        finally:
            lib.st_Buffer_delete(ptr)
        assert _objects(cb) == _objects(py)
        # and the Python re-encoding round-trips
        assert _objects(CBuffer.from_image(py.to_image())) == _objects(py)


def test_write_and_read_file(lib, tmp_path):
    e = lattices.fodo_ring()
    path = str(tmp_path / "fodo.bin")
    e.to_file(path)
    ptr = lib.st_Buffer_new_from_file(path.encode())
    try:
        out = str(tmp_path / "fodo2.bin")
        assert lib.st_Buffer_write_to_file(ptr, out.encode()) == 0
    finally:
        lib.st_Buffer_delete(ptr)
    assert _objects(CBuffer.fromfile(out)) == _objects(e.cbuffer)


def test_malformed_images_are_rejected(lib):
    img = lattices.fodo_ring().cbuffer.to_image().copy()
    bad = img.copy()
    bad[1] = 7  # size not a multiple of 8
    assert not lib.st_Buffer_new_on_data(bad.ctypes.data, bad.nbytes)
    bad = img.copy()
    bad[4] = 0  # objects section outside the buffer
    assert not lib.st_Buffer_new_on_data(bad.ctypes.data, bad.nbytes)
    assert _native.last_error()


def test_tracking_without_gpu_fails_loudly(lib):
    """No CPU fallback: on a machine without a GPU the free functions return
    failure and name the reason."""
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    e = lattices.fodo_ring()
    be = capi.c_buffer_from_image(e.cbuffer.to_image())
    q = lattices.gaussian_particles(4)
    blk = q.block.copy()
    sp = capi.particles_view(blk)
    st = lib.st_Track_all_particles_until_turn(C.byref(sp), be, 1)
    lib.st_Buffer_delete(be)
    assert st == -1
    assert "GPU" in _native.last_error() or "CUDA" in _native.last_error()
    assert np.array_equal(blk, q.block)


def test_line_density_link_survives_buffer_adoption():
    """A SCInterpolatedProfile linked to a LineDensityProfileData of the same
    buffer keeps pointing at it when the engine adopts the image at a new
    address (the field is a plain address, not a dataptr)."""
    import ctypes as C

    import numpy as np

    from sixtracklib_gb300 import CBuffer, _native
    from sixtracklib_gb300.beam_elements import Elements

    e = Elements()
    e.Drift(length=1.0)
    ld = len(e)
    e.LineDensityProfileData(values=np.linspace(1, 2, 8), z0=-1.0, dz=0.25, method="cubic")
    e.SCInterpolatedProfile(number_of_particles=1e10, length=1.0, line_density=ld)
    img = e.cbuffer.to_image()
    back = CBuffer.from_image(img)
    assert back.objects[2].links == [(6, ld)]
    lib = _native.load()
    buf = lib.st_Buffer_new_on_data(img.ctypes.data, img.nbytes)
    assert buf
    try:
        objs = [C.cast(lib.st_Buffer_get_const_object(buf, i), C.POINTER(C.c_uint64))
                for i in range(3)]
        ld_addr = int(objs[1][0])
        sc = C.cast(C.c_void_p(int(objs[2][0])), C.POINTER(C.c_uint64))
        assert int(sc[6]) == ld_addr != int(img[0])
    finally:
        lib.st_Buffer_delete(buf)



def test_node_queries_without_gpu(lib, capsys):
    """Node queries answer without a device: no CUDA node here, and no
    other architecture is served (trackjob.py:1215-1290)."""
    from sixtracklib_gb300.trackjob import TrackJob

    assert TrackJob.enabled_archs() == ["cuda"]
    assert TrackJob.num_available_nodes("opencl") == 0
    assert TrackJob.num_available_nodes() == 0
    assert TrackJob.num_available_nodes("cuda") == lib.st_CudaTrackJob_get_num_available_nodes()
    TrackJob.print_nodes("opencl")
    assert "no nodes" in capsys.readouterr().out
    assert lib.st_TrackJob_get_type_id(None) == -1
