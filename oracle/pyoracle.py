"""ctypes front-end for the CPU oracle and the reference build.

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg, never by the product package.

* ``Oracle()`` loads oracle/liboracle.so, the C restatement (oracle.c),
  compiling it first if needed;
* ``Oracle.reference()`` loads oracle/_ref/libstref.so, the reference's own
  tracking code built by oracle/build_ref.sh (only where the reference
  sources exist; None otherwise);
* ``Oracle.fast_policy(goertzel)`` loads oracle.c built with the CUDA
  engine's fast arithmetic in the plain-ring maps (``ORC_FAST_POLICY``),
  with the Goertzel kick for real-coefficient multipoles or with the Horner
  kick only: it measures on the CPU how far that policy departs from the
  reference.

Both expose identical calls on a CObjects lattice image (bytes / u64 array)
and a particle column block (21 x n u64 array, edited in place).
"""

from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libstref.so")
REF_OMP_LIB = os.path.join(HERE, "_ref", "libstref_omp.so")
# reference builds with other map feature flags (oracle/build_ref.sh):
# name -> (path, (bb4d, bb6d, spacecharge, tricub)), 2 enabled, 1 skip, 0 disabled
REF_FLAG_LIBS = {
    "a": (os.path.join(HERE, "_ref", "libstref_flags_a.so"), (1, 0, 1, 2)),
    "b": (os.path.join(HERE, "_ref", "libstref_flags_b.so"), (0, 1, 0, 1)),
}

CFLAGS = ["-O2", "-fPIC", "-shared", "-std=gnu99", "-fno-fast-math",
          "-ffp-contract=off", "-fopenmp"]


FAST_LIBS = {True: os.path.join(HERE, "liboracle_fast.so"),
             False: os.path.join(HERE, "liboracle_fast_horner.so")}


def _compile(lib: str, defines, force: bool) -> str:
    src = os.path.join(HERE, "oracle.c")
    newest = max(os.path.getmtime(src), os.path.getmtime(os.path.join(HERE, "oracle.h")))
    if not force and os.path.exists(lib) and os.path.getmtime(lib) >= newest:
        return lib
    tmp = lib + f".tmp{os.getpid()}"
    subprocess.check_call(["gcc", *CFLAGS, *defines, src, "-o", tmp, "-lm"])
    os.replace(tmp, lib)
    return lib


def build_oracle(force: bool = False) -> str:
    """Compile oracle.c into oracle/liboracle.so (gcc, no FMA contraction)."""
    return _compile(LIB, [], force)


def build_fast_policy(goertzel: bool = True, force: bool = False) -> str:
    """Compile oracle.c with the engine's fast arithmetic in the plain-ring
    maps (ORC_FAST_POLICY=1: Goertzel kick for real coefficients, 2: Horner
    kick only)."""
    return _compile(FAST_LIBS[goertzel], [f"-DORC_FAST_POLICY={1 if goertzel else 2}"], force)


def build_reference(ref_root: str | None = None) -> str | None:
    """Run oracle/build_ref.sh when the reference sources are present."""
    root = ref_root or os.environ.get("REF_ROOT", "/root/reference")
    if not os.path.exists(os.path.join(root, "sixtracklib/common/track/track.h")):
        return None
    env = dict(os.environ, REF_ROOT=root)
    subprocess.check_call(["bash", os.path.join(HERE, "build_ref.sh")], env=env,
                          stdout=subprocess.DEVNULL)
    return REF_LIB


def build_reference_cuda(ref_root: str | None = None) -> str | None:
    """Run oracle/build_ref_cuda.sh (the reference's CUDA kernels as an
    sm_103a cubin) when the reference sources are present and the cubin is
    missing or older than its recipe."""
    root = ref_root or os.environ.get("REF_ROOT", "/root/reference")
    if not os.path.exists(os.path.join(root, "sixtracklib/cuda/kernels/track_particles.cu")):
        return None
    out = os.path.join(HERE, "_ref", "ref_track_sm103a.cubin")
    deps = [os.path.join(HERE, f) for f in ("build_ref_cuda.sh", "ref_cuda_kernels.cu",
                                            "build_ref.sh")]
    if os.path.exists(out) and all(os.path.getmtime(out) >= os.path.getmtime(d) for d in deps):
        return out
    env = dict(os.environ, REF_ROOT=root)
    subprocess.check_call(["bash", os.path.join(HERE, "build_ref_cuda.sh")], env=env,
                          stdout=subprocess.DEVNULL)
    return out


class EbeConfig(C.Structure):
    _fields_ = [(n, C.c_int64) for n in (
        "order", "num_particles_to_store", "num_elements_to_store",
        "num_turns_to_store", "min_particle_id", "min_element_id", "min_turn",
        "max_particle_id", "max_element_id", "max_turn", "is_rolling")]


class MonitorOutputs(C.Structure):
    _fields_ = [("num", C.c_int64), ("cols", C.POINTER(C.c_void_p)),
                ("caps", C.POINTER(C.c_int64))]


def _u8(lattice):
    if isinstance(lattice, (bytes, bytearray)):
        arr = np.frombuffer(bytes(lattice), dtype=np.uint8)
    else:
        arr = np.ascontiguousarray(lattice).view(np.uint8)
    return arr


class Oracle:
    def __init__(self, path: str | None = None, prefix: str = "orc_"):
        if path is None:
            path = build_oracle()
        self.path = path
        self.lib = C.CDLL(path)
        self.prefix = prefix
        p = prefix
        vp, i64, u64 = C.c_void_p, C.c_int64, C.c_uint64
        self._until = getattr(self.lib, p + "track_until")
        self._until.argtypes = [vp, vp, i64, i64, i64, i64, vp]
        self._until.restype = C.c_int32
        self._line = getattr(self.lib, p + "track_line")
        self._line.argtypes = [vp, vp, i64, i64, i64, u64, u64, C.c_int, vp]
        self._line.restype = C.c_int32
        self._ebe = getattr(self.lib, p + "track_elem_by_elem")
        self._ebe.argtypes = [vp, vp, i64, i64, i64, vp, vp, i64, i64, vp]
        self._ebe.restype = C.c_int32
        self._ebe_idx = getattr(self.lib, p + "ebe_store_index")
        self._ebe_idx.argtypes = [vp, i64, i64, i64]
        self._ebe_idx.restype = C.c_int64
        self._cerrf = getattr(self.lib, p + "cerrf")
        self._cerrf.argtypes = [C.c_double, C.c_double, vp, vp]
        self._fields = getattr(self.lib, p + "fields_gauss")
        self._fields.argtypes = [C.c_double] * 5 + [C.c_int, vp, vp, vp, vp]
        if prefix == "orc_":
            self.lib.orc_set_aperture_mode.argtypes = [C.c_int, C.c_double,
                                                       C.c_double, C.c_double]

    @classmethod
    def fast_policy(cls, goertzel: bool = True):
        """The oracle with the engine's fast arithmetic in the plain-ring maps."""
        return cls(path=build_fast_policy(goertzel))

    @classmethod
    def reference(cls, omp: bool = False, flags: str | None = None):
        """The reference build; `flags` names one with other map feature
        flags (REF_FLAG_LIBS)."""
        path = REF_FLAG_LIBS[flags][0] if flags else (REF_OMP_LIB if omp else REF_LIB)
        if not os.path.exists(path):
            if build_reference() is None:
                return None
        return cls(path, prefix="ref_")

    # ------------------------------------------------------------ helpers
    @staticmethod
    def _mon(monitors):
        if not monitors:
            return None, None
        arrs = [np.ascontiguousarray(m) for m in monitors]
        cols = (C.c_void_p * len(arrs))(*[a.ctypes.data for a in arrs])
        caps = (C.c_int64 * len(arrs))(*[a.shape[-1] for a in arrs])
        mo = MonitorOutputs(len(arrs), cols, caps)
        return mo, (arrs, cols, caps)

    def set_num_threads(self, n: int) -> int:
        """Host threads of the oracle's particle loops; returns the number in use."""
        fn = self.lib.orc_set_num_threads
        fn.argtypes, fn.restype = [C.c_int], C.c_int
        return int(fn(int(n)))

    def set_aperture_mode(self, mode=2, min_length=0.0, x_limit=1.0, y_limit=1.0):
        self.lib.orc_set_aperture_mode(int(mode), float(min_length), float(x_limit),
                                       float(y_limit))

    def set_track_flags(self, bb4d=2, bb6d=2, spacecharge=2, tricub=0):
        """Map feature flags (2 enabled, 1 skip, 0 disabled); the defaults
        are the reference's default build."""
        fn = self.lib.orc_set_track_flags
        fn.argtypes = [C.c_int] * 4
        fn(int(bb4d), int(bb6d), int(spacecharge), int(tricub))

    def tricub_coefs(self, b):
        """The 64 tricubic coefficients (x^i y^j z^k at i + 4 j + 16 k) of
        one cell's 64 corner values."""
        b = np.ascontiguousarray(b, dtype=np.float64)
        out = np.empty(64)
        fn = getattr(self.lib, self.prefix + "tricub_coefs")
        fn.argtypes = [C.c_void_p, C.c_void_p]
        fn(b.ctypes.data, out.ctypes.data)
        return out

    def track_until(self, lattice, block, until_turn, i0=0, i1=None, monitors=None):
        lat = _u8(lattice)
        assert block.flags.c_contiguous and block.dtype.itemsize == 8
        n = block.shape[-1]
        i1 = n if i1 is None else i1
        mo, keep = self._mon(monitors)
        return self._until(lat.ctypes.data, block.ctypes.data, n, i0, i1,
                           int(until_turn), C.addressof(mo) if mo else None)

    def track_line(self, lattice, block, begin, end, finish_turn=False, i0=0,
                   i1=None, monitors=None):
        lat = _u8(lattice)
        n = block.shape[-1]
        i1 = n if i1 is None else i1
        mo, keep = self._mon(monitors)
        return self._line(lat.ctypes.data, block.ctypes.data, n, i0, i1, begin, end,
                          int(bool(finish_turn)), C.addressof(mo) if mo else None)

    def track_elem_by_elem(self, lattice, block, cfg: EbeConfig, out_block,
                           until_turn, i0=0, i1=None, monitors=None):
        lat = _u8(lattice)
        n = block.shape[-1]
        i1 = n if i1 is None else i1
        mo, keep = self._mon(monitors)
        out_ptr = out_block.ctypes.data if out_block is not None else None
        out_n = out_block.shape[-1] if out_block is not None else 0
        return self._ebe(lat.ctypes.data, block.ctypes.data, n, i0, i1,
                         C.addressof(cfg), out_ptr, out_n, int(until_turn),
                         C.addressof(mo) if mo else None)

    def ebe_store_index(self, cfg, pid, elem, turn):
        return self._ebe_idx(C.addressof(cfg), pid, elem, turn)

    def cerrf_n(self, re, im):
        """w(z) of arrays (the oracle's cerrf, element by element)."""
        re = np.ascontiguousarray(re, dtype=np.float64)
        im = np.ascontiguousarray(im, dtype=np.float64)
        wr, wi = np.empty_like(re), np.empty_like(re)
        fn = self.lib.orc_cerrf_n
        fn.argtypes = [C.c_void_p] * 4 + [C.c_int64]
        fn(re.ctypes.data, im.ctypes.data, wr.ctypes.data, wi.ctypes.data, re.size)
        return wr, wi

    def cerrf(self, re, im):
        a, b = C.c_double(), C.c_double()
        self._cerrf(float(re), float(im), C.byref(a), C.byref(b))
        return a.value, b.value

    def fields_gauss(self, x, y, sx, sy, msd, skip_gs):
        v = [C.c_double() for _ in range(4)]
        self._fields(x, y, sx, sy, msd, int(skip_gs), *[C.byref(t) for t in v])
        return tuple(t.value for t in v)
