"""Output-buffer planning of the C ABI (st_OutputBuffer_*, the beam-monitor
and elem-by-elem output helpers) against the reference's own host code:
output/output_buffer.c with the helpers it calls, compiled from the
reference sources into oracle/_ref/libstref_output.so by
oracle/build_ref.sh.  Both libraries get the same lattices and particle
sets (written by this engine, loaded by each through its own
st_Buffer_new_from_file); flags, sizes, offsets, the output buffers'
Particles blocks, the monitors' fields and the assigned output addresses
must agree.  The reference library runs alone in a spawned child process:
in a process that has also run the engine's library and many other
calls, its st_OutputBuffer_prepare now and then fails on inputs it
handles in a fresh process.  Nothing here needs a GPU."""

import multiprocessing

import ctypes as C
import os

import numpy as np
import pytest

from sixtracklib_gb300 import _native

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.path.join(os.path.dirname(HERE), "oracle", "_ref", "libstref_output.so")

D, I64, U64, U32, VP, B = C.c_double, C.c_int64, C.c_uint64, C.c_uint32, C.c_void_p, C.c_bool
P64 = C.POINTER(C.c_uint64)


class Particles(C.Structure):
    _fields_ = [("num_particles", I64)] + [(f"r{k}", C.POINTER(D)) for k in range(17)] + [
        ("particle_id", C.POINTER(I64)), ("at_element_id", C.POINTER(I64)),
        ("at_turn", C.POINTER(I64)), ("state", C.POINTER(I64))]


class EbeConfig(C.Structure):
    _fields_ = [(n, I64) for n in (
        "order", "num_particles_to_store", "num_elements_to_store", "num_turns_to_store",
        "min_particle_id", "min_element_id", "min_turn", "max_particle_id", "max_element_id",
        "max_turn", "is_rolling")] + [("out_store_addr", U64)]


EBE_GETTERS = ("order", "num_particles_to_store", "num_elements_to_store",
               "num_turns_to_store", "out_store_num_particles", "min_particle_id",
               "max_particle_id", "min_element_id", "max_element_id", "min_turn", "max_turn")

COMMON = {
    "st_Buffer_new": ([U64], VP), "st_Buffer_delete": ([VP], None),
    "st_Buffer_new_from_file": ([C.c_char_p], VP),
    "st_OutputBuffer_requires_output_buffer_ext": ([U32], B),
    "st_OutputBuffer_requires_elem_by_elem_output_ext": ([U32], B),
    "st_OutputBuffer_requires_beam_monitor_output_ext": ([U32], B),
    "st_OutputBuffer_required_for_tracking": ([VP, VP, U64], U32),
    "st_OutputBuffer_required_for_tracking_of_particle_sets": ([VP, U64, VP, VP, U64], U32),
    "st_OutputBuffer_calculate_output_buffer_params": ([VP, VP, U64] + [VP] * 4 + [U64], I64),
    "st_OutputBuffer_calculate_output_buffer_params_for_particles_sets":
        ([VP, VP, U64, VP, U64] + [VP] * 4 + [U64], I64),
    "st_OutputBuffer_prepare": ([VP, VP, VP, U64, VP, VP, VP], I64),
    "st_OutputBuffer_prepare_for_particle_sets": ([VP, VP, VP, U64, VP, U64, VP, VP, VP], I64),
    "st_BeamMonitor_assign_output_buffer": ([VP, VP, I64, U64], I64),
    "st_BeamMonitor_assign_output_buffer_from_offset": ([VP, VP, I64, U64], I64),
    "st_BeamMonitor_calculate_output_buffer_params": ([VP, VP] + [VP] * 4 + [U64], I64),
    "st_BeamMonitor_prepare_output_buffer": ([VP, VP, VP, VP], I64),
    "st_ElemByElemConfig_assign_output_buffer": ([VP, VP, U64], I64),
    "st_ElemByElemConfig_create": ([], VP), "st_ElemByElemConfig_delete": ([VP], None),
    "st_ElemByElemConfig_preset_ext": ([VP], VP), "st_ElemByElemConfig_clear_ext": ([VP], None),
    "st_ElemByElemConfig_is_active_ext": ([VP], B),
    "st_ElemByElemConfig_is_rolling_ext": ([VP], B),
    "st_ElemByElemConfig_get_output_store_address_ext": ([VP], U64),
    "st_ElemByElemConfig_set_order_ext": ([VP, I64], None),
    "st_ElemByElemConfig_set_is_rolling_ext": ([VP, B], None),
    "st_ElemByElemConfig_set_output_store_address_ext": ([VP, U64], None),
    **{f"st_ElemByElemConfig_get_{f}_ext": ([VP], I64) for f in EBE_GETTERS},
    "st_ElemByElemConfig_get_order_ext": ([VP], C.c_int32),  # an enum
}
OURS = {"st_Buffer_get_num_of_objects": ([VP], U64),
        "st_Buffer_get_const_object": ([VP, U64], VP),
        "st_Buffer_write_to_file": ([VP, C.c_char_p], C.c_int32),
        "st_Particles_new": ([VP, U64], VP),
        "st_Particles_buffer_get_particles": ([VP, U64], VP),
        "st_Particles_buffer_get_total_num_of_particles": ([VP], U64),
        "st_Particles_calculate_difference": ([VP, VP, VP], None),
        "st_Drift_add": ([VP, D], VP), "st_Cavity_add": ([VP, D, D, D], VP),
        "st_BeamMonitor_add": ([VP, I64, I64, I64, U64, I64, I64, B, B], VP)}
THEIRS = {"st_Buffer_new_detailed": ([U64] * 5, VP),
          "st_Buffer_get_num_of_objects_ext": ([VP], U64),
          "st_Buffer_get_objects_begin_addr_ext": ([VP], U64),
          "st_Particles_buffer_get_particles_ext": ([VP, U64], VP),
          "st_Particles_buffer_get_total_num_of_particles_ext": ([VP], U64),
          "st_Particles_calculate_difference_ext": ([VP, VP, VP], None)}


def _bind(lib, table):
    for name, (args, res) in table.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res


# The status the two libraries return is an int (ours int32, the
# reference's int / arch status): compare the low 32 bits, signed.
def _st(v):
    return C.c_int32(v & 0xFFFFFFFF).value


class Side:
    """One library (the engine's or the reference's) behind one interface."""

    def __init__(self, lib, ours):
        self.L, self.ours = lib, ours

    def new_output(self):
        """An empty output buffer.  The reference's is made at full size up
        front (as its own Python layer does before st_OutputBuffer_prepare):
        appending to its st_Buffer_new(0) buffer succeeds or fails depending
        on the allocator's history in this process."""
        if self.ours:
            return self.L.st_Buffer_new(0)
        return self.L.st_Buffer_new_detailed(64, 1 << 18, 64 * 21, 0, 0x10000)  # mempool store

    def load(self, path):
        b = self.L.st_Buffer_new_from_file(str(path).encode())
        assert b
        return b

    def objects(self, b):
        if self.ours:
            n = self.L.st_Buffer_get_num_of_objects(b)
            return [tuple(C.cast(self.L.st_Buffer_get_const_object(b, i), P64)[k] for k in range(3))
                    for i in range(n)]
        n = self.L.st_Buffer_get_num_of_objects_ext(b)
        t = C.cast(C.c_void_p(self.L.st_Buffer_get_objects_begin_addr_ext(b)), P64)
        return [(t[3 * i], t[3 * i + 1], t[3 * i + 2]) for i in range(n)]

    def particles(self, b, i):
        fn = (self.L.st_Particles_buffer_get_particles if self.ours
              else self.L.st_Particles_buffer_get_particles_ext)
        return fn(b, i)

    def layout(self, out):
        """(type id, particle count) per object of an output buffer."""
        return [(t, C.cast(C.c_void_p(a), C.POINTER(I64))[0] if t == 1 else None)
                for a, t, _ in self.objects(out)]

    def monitors(self, eb, out=None):
        """Every monitor's fields; its output address as an object index of
        `out` (-1 for none)."""
        where = {a: i for i, (a, _, _) in enumerate(self.objects(out))} if out else {}
        rows = []
        for a, t, _ in self.objects(eb):
            if t != 10:
                continue
            w = list(C.cast(C.c_void_p(a), C.POINTER(I64))[0:9])
            w[3] = where.get(w[3] & 0xFFFFFFFFFFFFFFFF, -1 if w[3] == 0 else -2)
            rows.append(tuple(w))
        return rows


def _ref_side():
    ref = C.CDLL(REF)
    _bind(ref, {**COMMON, **THEIRS})
    return Side(ref, False)


@pytest.fixture(scope="module")
def ours():
    if not os.path.exists(REF):
        pytest.skip("reference output-buffer library not built (oracle/build_ref.sh)")
    _native.load()
    lib = C.CDLL(_native.lib_path())
    _bind(lib, {**COMMON, **OURS})
    return Side(lib, True)


def _particles(L, buf, pid, elem, turn):
    p = C.cast(L.st_Particles_new(buf, len(pid)), C.POINTER(Particles)).contents
    for k in range(len(pid)):
        p.particle_id[k], p.at_element_id[k], p.at_turn[k], p.state[k] = pid[k], elem[k], turn[k], 1
        for c in range(17):
            getattr(p, f"r{c}")[k] = 0.25 * k + c


def _lattice(L, kind, b):
    mon = lambda n, start, skip, rolling=False: L.st_BeamMonitor_add(  # noqa: E731
        b, n, start, skip, 0, 0, 0, rolling, False)
    if kind == "leading_particles":  # a non-element object shifts the element ids
        _particles(L, b, [0], [0], [0])
    if kind != "no_monitors":
        L.st_Drift_add(b, 1.0)
        mon(3, 0, 1)
        L.st_Drift_add(b, 2.0)
        mon(2, 5, 2)
        mon(0, 0, 1)           # stores nothing
        mon(4, 1, 2, True)     # rolling, starts before turn 2
        mon(5, 0, 2)           # started before turn 2, stores left
        L.st_Cavity_add(b, 1e6, 4e8, 180.0)
    else:
        for k in range(4):
            L.st_Drift_add(b, 1.0 + k)


PSETS = {
    "plain": [([0, 1, 2, 3, 4], [0] * 5, [0] * 5)],
    "turns_and_ids": [([3, -5, 7, 4, 9, 6, 8], [0, 2, 1, 0, 3, 0, 0], [2, 2, 3, 2, 4, 2, 2])],
    "two_sets": [([2, 3, 4], [0, 1, 0], [1, 1, 1]), ([10, 11], [0, 0], [3, 1])],
}


@pytest.fixture(scope="module")
def files(ours, tmp_path_factory):
    L = ours.L
    d = tmp_path_factory.mktemp("outbuf")
    builds = {kind: (lambda b, k=kind: _lattice(L, k, b))
              for kind in ("monitors", "leading_particles", "no_monitors")}
    for name, sets in PSETS.items():
        builds[name] = lambda b, sets=sets: [_particles(L, b, *x) for x in sets]
    builds["empty"] = lambda b: None
    builds["only_particles"] = lambda b: _particles(L, b, [0], [0], [0])
    builds["no_particles"] = lambda b: L.st_Drift_add(b, 1.0)
    out = {}
    for name, build in builds.items():
        b = L.st_Buffer_new(0)
        build(b)
        out[name] = str(d / f"{name}.bin")
        assert L.st_Buffer_write_to_file(b, out[name].encode()) == 0
        L.st_Buffer_delete(b)
    return out


UNTIL = (0, 1, 2, 3, 6)
CASES = [(lat, ps) for lat in ("monitors", "leading_particles", "no_monitors")
         for ps in PSETS]


def _sizes(side, fn, *args):
    n = [C.c_uint64(0xDEAD) for _ in range(4)]
    rc = fn(*args[:-1], *[C.byref(x) for x in n], args[-1])
    return _st(rc), tuple(x.value for x in n) if _st(rc) == 0 else None


def _prepare(s, files, lattice, pset, until, sets):
    L = s.L
    eb, pb, out = s.load(files[lattice]), s.load(files[pset]), s.new_output()
    ebe, mon, turn = C.c_uint64(77), C.c_uint64(77), C.c_int64(77)
    if sets:
        idx = (C.c_uint64 * len(PSETS[pset]))(*range(len(PSETS[pset])))
        rc = L.st_OutputBuffer_prepare_for_particle_sets(eb, out, pb, len(idx), idx, until,
                                                         C.byref(ebe), C.byref(mon),
                                                         C.byref(turn))
    else:
        rc = L.st_OutputBuffer_prepare(eb, out, s.particles(pb, 0), until, C.byref(ebe),
                                       C.byref(mon), C.byref(turn))
    res = [_st(rc), ebe.value, mon.value, turn.value, s.layout(out), s.monitors(eb)]
    # the monitors' own preparation, on a second output buffer
    out2, off = s.new_output(), C.c_uint64(77)
    res.append(_st(L.st_BeamMonitor_prepare_output_buffer(eb, out2, s.particles(pb, 0),
                                                          C.byref(off))))
    res += [off.value, s.layout(out2), s.monitors(eb)]
    L.st_Buffer_delete(out2)
    if _st(rc) == 0:
        res.append(_st(L.st_BeamMonitor_assign_output_buffer(eb, out, turn.value, until)))
        res.append(s.monitors(eb, out))
        res.append(_st(L.st_BeamMonitor_assign_output_buffer_from_offset(eb, out, turn.value,
                                                                          ebe.value + 1)))
        cfg = EbeConfig()
        res.append(_st(L.st_ElemByElemConfig_assign_output_buffer(C.byref(cfg), out, 0)))
        where = {a: i for i, (a, _, _) in enumerate(s.objects(out))}
        res.append(where.get(cfg.out_store_addr, -1))
    for b in (eb, pb, out):
        L.st_Buffer_delete(b)
    return res


def _flags(s, files, lattice, pset):
    L = s.L
    eb, pb = s.load(files[lattice]), s.load(files[pset])
    p = s.particles(pb, 0)
    idx = (C.c_uint64 * len(PSETS[pset]))(*range(len(PSETS[pset])))
    row = []
    for until in UNTIL:
        row.append(L.st_OutputBuffer_required_for_tracking(p, eb, until))
        row.append(L.st_OutputBuffer_required_for_tracking_of_particle_sets(
            pb, len(idx), idx, eb, until))
        row.append(_sizes(s, L.st_OutputBuffer_calculate_output_buffer_params, eb, p, until, 8))
        row.append(_sizes(s, L.st_OutputBuffer_calculate_output_buffer_params_for_particles_sets,
                          eb, pb, len(idx), idx, until, 8))
    row.append(_sizes(s, L.st_BeamMonitor_calculate_output_buffer_params, eb, p, 8))
    L.st_Buffer_delete(eb)
    L.st_Buffer_delete(pb)
    return row


def _failures(s, files):
    """An empty lattice, a lattice of particles only and a particles buffer
    without a Particles object."""
    L = s.L
    row = []
    for lat, ps in (("empty", "plain"), ("only_particles", "plain"),
                    ("monitors", "no_particles")):
        eb, pb, out = s.load(files[lat]), s.load(files[ps]), s.new_output()
        p = s.particles(pb, 0)
        row.append(_sizes(s, L.st_OutputBuffer_calculate_output_buffer_params, eb, p, 2, 8))
        row.append(_st(L.st_OutputBuffer_prepare(eb, out, p, 2, None, None, None)))
        row.append(L.st_OutputBuffer_required_for_tracking(p, eb, 2))
        for b in (eb, pb, out):
            L.st_Buffer_delete(b)
    return row


def _particle_helpers(s, files):
    L = s.L
    total_fn = (L.st_Particles_buffer_get_total_num_of_particles if s.ours
                else L.st_Particles_buffer_get_total_num_of_particles_ext)
    diff_fn = (L.st_Particles_calculate_difference if s.ours
               else L.st_Particles_calculate_difference_ext)
    pb, diff_buf, other = (s.load(files[n]) for n in ("two_sets", "two_sets", "turns_and_ids"))
    a, d = s.particles(pb, 0), s.particles(diff_buf, 0)
    diff_fn(a, a, d)
    dp = C.cast(d, C.POINTER(Particles)).contents
    zero = [dp.r6[k] for k in range(3)] + [dp.particle_id[k] for k in range(3)]
    before = [dp.r0[k] for k in range(3)]
    diff_fn(a, s.particles(other, 0), d)  # 3 against 7 particles: diff stays
    after = [dp.r0[k] for k in range(3)]
    res = (total_fn(pb), zero, before == after)
    for b in (pb, diff_buf, other):
        L.st_Buffer_delete(b)
    return res


def _ebe_accessors(s):
    """Every accessor of the elem-by-elem configuration over create, preset,
    set, clear and a hand-filled configuration (the struct layouts agree)."""
    L = s.L

    def read(c):
        return ([L.st_ElemByElemConfig_is_active_ext(c), L.st_ElemByElemConfig_is_rolling_ext(c),
                 L.st_ElemByElemConfig_get_output_store_address_ext(c)] +
                [getattr(L, f"st_ElemByElemConfig_get_{f}_ext")(c) for f in EBE_GETTERS] +
                [bytes(C.string_at(c, C.sizeof(EbeConfig)))])

    rows = []
    c = L.st_ElemByElemConfig_create()
    rows.append(read(c))
    L.st_ElemByElemConfig_set_order_ext(c, 0)
    L.st_ElemByElemConfig_set_is_rolling_ext(c, False)
    L.st_ElemByElemConfig_set_output_store_address_ext(c, 4096)
    rows.append(read(c))
    cfg = EbeConfig(0, 3, 4, 5, 2, 1, 7, 4, 4, 11, 0, 8192)
    rows.append(read(C.byref(cfg)))
    L.st_ElemByElemConfig_clear_ext(C.byref(cfg))
    rows.append(read(C.byref(cfg)))
    rows.append(L.st_ElemByElemConfig_preset_ext(C.byref(cfg)) == C.addressof(cfg))
    rows.append(read(C.byref(cfg)))
    L.st_ElemByElemConfig_delete(c)
    rows.append((L.st_ElemByElemConfig_is_active_ext(None),
                 L.st_ElemByElemConfig_preset_ext(None)))
    return rows


def _all_results(s, files):
    """Every comparison of this file, for one library."""
    out = {("flags", lat, ps): _flags(s, files, lat, ps) for lat, ps in CASES}
    for lat, ps in CASES:
        for until in UNTIL:
            for sets in (False, True):
                out[("prepare", lat, ps, until, sets)] = _prepare(s, files, lat, ps, until, sets)
    out[("failures",)] = _failures(s, files)
    out[("predicates",)] = [(s.L.st_OutputBuffer_requires_output_buffer_ext(f),
                             s.L.st_OutputBuffer_requires_elem_by_elem_output_ext(f),
                             s.L.st_OutputBuffer_requires_beam_monitor_output_ext(f))
                            for f in range(4)]
    out[("particles",)] = _particle_helpers(s, files)
    out[("ebe_accessors",)] = _ebe_accessors(s)
    return out


def _reference_results(files):
    """Runs in the spawned child: the reference library alone."""
    return _all_results(_ref_side(), files)


@pytest.fixture(scope="module")
def results(ours, files):
    mine = _all_results(ours, files)
    with multiprocessing.get_context("spawn").Pool(1) as pool:
        theirs = pool.apply(_reference_results, (files,))
    return mine, theirs


@pytest.mark.parametrize("lattice,pset", CASES)
def test_flags_and_sizes_match_the_reference(results, lattice, pset):
    mine, theirs = (r[("flags", lattice, pset)] for r in results)
    assert mine == theirs
    if lattice != "no_monitors":  # something was actually planned
        assert any(isinstance(r, tuple) and r[0] == 0 and r[1] and r[1][0] > 0 for r in mine)


@pytest.mark.parametrize("sets", [False, True])
@pytest.mark.parametrize("until", UNTIL)
@pytest.mark.parametrize("lattice,pset", CASES)
def test_prepare_and_assign_match_the_reference(results, lattice, pset, until, sets):
    mine, theirs = (r[("prepare", lattice, pset, until, sets)] for r in results)
    assert mine == theirs


def test_prepare_lays_out_the_expected_blocks(results):
    """The layout itself, for one case: the elem-by-elem block first
    (5 particles x 8 elements x 3 turns), then one block per monitor that
    starts at or after turn 0 and stores something (5 ids x num_stores)."""
    mine = results[0][("prepare", "monitors", "plain", 3, False)]
    rc, ebe, mon, turn, layout = mine[:5]
    assert (rc, ebe, mon, turn) == (0, 0, 1, 0)
    assert layout == [(1, 5 * 8 * 3), (1, 5 * 3), (1, 5 * 2), (1, 5 * 4), (1, 5 * 5)]
    assert mine[10] == 0  # monitors assigned: blocks 1..4 in lattice order
    assert [m[3] for m in mine[11]] == [1, 2, -1, 3, 4]


def test_failures_match_the_reference(results):
    mine, theirs = (r[("failures",)] for r in results)
    assert mine == theirs
    assert mine[1] == -1 and mine[4] == -1 and mine[7] == -1


def test_flag_predicates_match_the_reference(results):
    mine, theirs = (r[("predicates",)] for r in results)
    assert mine == theirs == [(f != 0, bool(f & 1), bool(f & 2)) for f in range(4)]


def test_particle_helpers_match_the_reference(results):
    mine, theirs = (r[("particles",)] for r in results)
    assert mine == theirs
    assert mine[0] == 5 and mine[1] == [0.0] * 3 + [0] * 3 and mine[2]


def test_elem_by_elem_accessors_match_the_reference(results):
    mine, theirs = (r[("ebe_accessors",)] for r in results)
    assert mine == theirs
    assert mine[2][0] is True and mine[3][0] is False  # filled: active; cleared: not
