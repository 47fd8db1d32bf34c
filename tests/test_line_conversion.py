"""Lattice input conversions on the CPU: thin MAD-X sequences
(``Elements.from_mad``, python/sixtracklib/mad_helper.py), pysixtrack-style
lines (``Elements.from_line`` / ``append_line``), the element converter
(python/sixtracklib/pysixtrack_helper.py) and the in-place strength setters
that the reference's tests/python/beam_elements/test_multipole.py uses.

Neither cpymad nor pysixtrack is installed: the inputs are small stand-in
objects with the attributes those packages' objects have.
"""

from math import factorial
from types import SimpleNamespace

import numpy as np
import pytest

from sixtracklib_gb300.beam_elements import (Q_PART_NAMED, BeamBeam6D, Elements, bb6d_data)


# ------------------------------------------------------------ MAD-X stand-ins
def _mad_el(kind, **attrs):
    return SimpleNamespace(base_type=SimpleNamespace(name=kind), length=attrs.pop("length", 0.0),
                           **attrs)


class _Sequence:
    def __init__(self, items):
        self._items = items  # (name, position, element)
        self.elements = [el for _, _, el in items]

    def element_names(self):
        return [n for n, _, _ in self._items]

    def element_positions(self):
        return [p for _, p, _ in self._items]


def _thin_sequence():
    return _Sequence([
        ("start", 0.0, _mad_el("marker")),
        ("qf", 1.5, _mad_el("multipole", knl=[0.0, 0.05, 0.2], ksl=[0.0, 1e-3], lrad=0.3)),
        ("bpm", 1.5, _mad_el("monitor")),
        ("hk", 3.0, _mad_el("hkicker", kick=2e-5, lrad=0.1)),
        ("vk", 3.25, _mad_el("vkicker", kick=-3e-5, lrad=0.0)),
        ("cav", 7.0, _mad_el("rfcavity", volt=2.5, freq=400.8, lag=0.5)),
        ("dip", 9.0, _mad_el("multipole", knl=[1e-3], lrad=1.0)),
        ("end", 9.0, _mad_el("marker")),
    ])


def test_from_mad_thin_sequence():
    e = Elements.from_mad(_thin_sequence())
    objs = e.get_elements()
    kinds = [type(o).__name__ for o in objs]
    assert kinds == ["Drift", "Drift", "Multipole", "Drift", "Drift", "Multipole", "Drift",
                     "Multipole", "Drift", "Cavity", "Drift", "Multipole", "Drift"]
    # gaps become drifts, markers and monitors zero-length drifts
    assert [o.length for o in objs if type(o).__name__ == "Drift"] == \
        [0.0, 1.5, 0.0, 1.5, 0.25, 3.75, 2.0, 0.0]
    qf = objs[2]
    assert qf.order == 2 and qf.length == 0.3 and qf.hxl == 0.0 and qf.hyl == 0.0
    np.testing.assert_array_equal(qf.knl, [0.0, 0.05, 0.2])
    np.testing.assert_array_equal(qf.ksl, [0.0, 1e-3, 0.0])
    hk, vk = objs[5], objs[7]
    np.testing.assert_array_equal(hk.knl, [-2e-5])
    np.testing.assert_array_equal(vk.ksl, [-3e-5])
    assert hk.length == 0.1
    cav = objs[9]
    assert (cav.voltage, cav.frequency, cav.lag) == (2.5e6, 400.8e6, 180.0)
    dip = objs[11]  # hxl = knl[0] for a MAD-X multipole
    assert dip.hxl == 1e-3 and dip.length == 1.0
    np.testing.assert_array_equal(dip.ksl, [0.0])


def test_from_mad_exact_drift_and_errors():
    e = Elements.from_mad(_thin_sequence(), exact_drift=True)
    kinds = {type(o).__name__ for o in e.get_elements()}
    assert "Drift" not in kinds and "DriftExact" in kinds
    thick = _Sequence([("q", 1.0, _mad_el("quadrupole", length=0.5, k1=0.1))])
    with pytest.raises(ValueError, match="length > 0"):
        Elements.from_mad(thick)
    other = _Sequence([("s", 1.0, _mad_el("solenoid"))])
    with pytest.raises(AttributeError):
        Elements.from_mad(other)


# ------------------------------------------------------- pysixtrack stand-ins
def _line_el(cls_name, **fields):
    cls = type(cls_name, (), {
        "to_dict": lambda self, keepextra=False: dict(fields, **({"extra": 1} if keepextra else {})),
        "as_dict": lambda self: dict(fields)})
    return cls()


def test_from_line_matches_direct_construction():
    z = np.array([-0.05, 0.0, 0.05])
    bb6d = dict(phi=1e-3, alpha=0.3, x_bb_co=1e-6, y_bb_co=-2e-6, charge_slices=[1e10] * 3,
                zeta_slices=z, sigma_11=1e-6, sigma_12=0.0, sigma_13=0.0, sigma_14=0.0,
                sigma_22=4e-6, sigma_23=0.0, sigma_24=0.0, sigma_33=1.2e-6, sigma_34=0.0,
                sigma_44=3e-6, x_co=0.0, px_co=0.0, y_co=0.0, py_co=0.0, zeta_co=0.0,
                delta_co=0.0, min_sigma_diff=1e-10, threshold_singular=1e-28, d_x=0.0,
                d_px=0.0, d_y=0.0, d_py=0.0, d_zeta=0.0, d_delta=0.0, enabled=1.0)
    bb4d = dict(charge=1e11, sigma_x=1e-3, sigma_y=1.2e-3, beta_r=1.0, min_sigma_diff=1e-10,
                x_bb=1e-5, y_bb=0.0, d_px=0.0, d_py=0.0, enabled=1.0)
    line = SimpleNamespace(elements=[
        _line_el("Drift", length=1.25),
        _line_el("Multipole", knl=[0.0, 0.05, 0.3], ksl=[0.0, 0.0, 1e-2], hxl=0.0, hyl=0.0,
                 length=0.0),
        _line_el("SRotation", angle=2.5),
        _line_el("XYShift", dx=1e-5, dy=-2e-5),
        _line_el("Cavity", voltage=6e6, frequency=400e6, lag=180.0),
        _line_el("RFMultipole", voltage=1e5, frequency=400e6, lag=30.0, knl=[1e-6, 1e-3],
                 ksl=[0.0, 2e-4], pn=[10.0, 20.0], ps=[5.0, 0.0]),
        _line_el("BeamBeam4D", **bb4d),
        _line_el("BeamBeam6D", **bb6d),
        _line_el("DriftExact", length=0.5),
    ])
    got = Elements.from_line(line)
    ref = Elements()
    ref.Drift(length=1.25)
    ref.Multipole(knl=[0.0, 0.05, 0.3], ksl=[0.0, 0.0, 1e-2])
    ref.SRotation(angle=2.5)
    ref.XYShift(dx=1e-5, dy=-2e-5)
    ref.Cavity(voltage=6e6, frequency=400e6, lag=180.0)
    ref.RFMultipole(voltage=1e5, frequency=400e6, lag=30.0, knl=[1e-6, 1e-3], ksl=[0.0, 2e-4],
                    pn=[10.0, 20.0], ps=[5.0, 0.0])
    ref.BeamBeam4D(data=[Q_PART_NAMED, 1e11, 1e-3, 1.2e-3, 1.0, 1e-10, 1e-5, 0.0, 0.0, 0.0, 1.0])
    ref.BeamBeam6D(data=bb6d_data(
        Q_PART_NAMED, 1e-3, 0.3, 1e-6, -2e-6, [1e10] * 3, z,
        (1e-6, 0.0, 0.0, 0.0, 4e-6, 0.0, 0.0, 1.2e-6, 0.0, 3e-6)))
    ref.DriftExact(length=0.5)
    assert np.array_equal(got.cbuffer.to_image(), ref.cbuffer.to_image())
    # append_line extends an existing lattice
    n = len(got)
    got.append_line(SimpleNamespace(elements=[_line_el("Drift", length=2.0)]))
    assert len(got) == n + 1 and got.get(n).length == 2.0
    assert set(got.gen_builder()) == set(Elements.element_types)


def test_strength_setters_write_the_buffer():
    """As the reference's test_multipole.py: random knl / ksl up to order 9,
    bal = k / n!, then set_knl / set_ksl on the lattice's elements."""
    rng = np.random.default_rng(0)
    e = Elements()
    data = []
    for _ in range(64):
        order = int(rng.integers(0, 10))
        knl = rng.uniform(0.0, 100.0, order + 1)
        ksl = rng.uniform(0.0, 100.0, order + 1)
        e.Multipole(knl=knl, ksl=ksl)
        data.append((order, knl, ksl))
    image0 = e.cbuffer.to_image().copy()
    for i, (order, knl, ksl) in enumerate(data):
        m = e.get(i)
        assert m.order == order
        np.testing.assert_allclose(m.knl, knl, rtol=1e-15)
        bal = np.zeros(2 * order + 2)
        bal[0::2] = [k / factorial(j) for j, k in enumerate(knl)]
        bal[1::2] = [k / factorial(j) for j, k in enumerate(ksl)]
        np.testing.assert_allclose(m.bal, bal, rtol=1e-15)
        for j in range(order + 1):
            kn, ks = rng.uniform(0.0, 100.0, 2)
            m.set_knl(kn, j)
            m.set_ksl(ks, j)
            knl[j], ksl[j] = kn, ks
    assert not np.array_equal(e.cbuffer.to_image(), image0)  # the image follows
    for i, (order, knl, ksl) in enumerate(data):
        np.testing.assert_allclose(e.get(i).knl, knl, rtol=1e-15)
        np.testing.assert_allclose(e.get(i).ksl, ksl, rtol=1e-15)
    r = Elements()
    r.RFMultipole(voltage=1.0, frequency=2.0, lag=3.0, knl=np.array([1.0, 2.0]), pn=[10.0, 20.0])
    rf = r.get(0)
    rf.set_ps(5.0, 1)
    rf.set_knl(4.0, 1)
    np.testing.assert_array_equal(r.get(0).ps, [0.0, 5.0])
    np.testing.assert_array_equal(r.get(0).pn, [10.0, 20.0])
    np.testing.assert_array_equal(r.get(0).knl, [1.0, 4.0])
    with pytest.raises(AssertionError):
        rf.set_knl(1.0, 2)


def test_element_converter():
    from sixtracklib_gb300.beam_elements import BeamBeam4D, Drift, Multipole
    from sixtracklib_gb300.pysixtrack_helper import BeamElementConverter as C

    assert C.get_elemtype(4) is Multipole and C.get_elemtype(9) is None
    assert C.get_typeid.__func__(Drift) == 2 and C.get_typeid.__func__(BeamBeam4D) == 8
    e = Elements()
    m = C.from_pysixtrack(_line_el("Multipole", knl=[0.0, 0.1], ksl=[0.0, 0.0], hxl=0.0,
                                   hyl=0.0, length=0.0), cbuffer=e.cbuffer)
    assert isinstance(m, Multipole) and len(e) == 1
    np.testing.assert_array_equal(e.get(0).knl, [0.0, 0.1])
    assert C.from_pysixtrack(_line_el("Solenoid", ks=1.0)) is None
    if not C.available():
        with pytest.raises(ImportError):
            C.to_pysixtrack(e.get(0))


def test_bb6d_named_parameters_need_all_fields():
    with pytest.raises(KeyError):
        BeamBeam6D(x_bb_co=0.0, phi=0.0)


def test_tricub_elements_round_trip(oracle):
    """TriCubData / TriCub (python/sixtracklib/tricub.py) encode and decode;
    the map is compiled out, so tracking through the lattice fails, as in
    the reference's default build."""
    from sixtracklib_gb300 import lattices
    from sixtracklib_gb300.beam_elements import TriCub, TriCubData
    from sixtracklib_gb300.cbuffer import CBuffer

    e = Elements()
    e.Drift(length=1.0)
    table = np.arange(2 * 3 * 4 * 8, dtype=np.float64) * 0.5
    e.TriCubData(x0=-1.0, dx=0.5, nx=2, y0=-2.0, dy=0.25, ny=3, z0=0.0, dz=0.1, nz=4,
                 mirror_x=1, table_addr=table)
    e.TriCub(x_shift=1e-3, length=0.2, data_addr=0)
    back = Elements(cbuffer=CBuffer.from_image(e.cbuffer.to_image()))
    d, t = back.get(1), back.get(2)
    assert isinstance(d, TriCubData) and isinstance(t, TriCub)
    assert (d.nx, d.ny, d.nz, d.mirror_x, d.dy) == (2, 3, 4, 1, 0.25)
    np.testing.assert_array_equal(d.table_addr, table)
    assert (t.x_shift, t.length) == (1e-3, 0.2) and TriCub.data_addr_offset() == 56
    p = lattices.gaussian_particles(8, seed=1).block.copy()
    assert oracle.track_until(e.cbuffer.to_image(), p, 1) == -1


def test_truncated_objects_stay_undecoded():
    """An object shorter than its type's struct (a malformed or placeholder
    entry) is returned as the raw CObject instead of being decoded."""
    from sixtracklib_gb300.autodiff import parameter_table
    from sixtracklib_gb300.beam_elements import TYPE_TRICUB
    from sixtracklib_gb300.cbuffer import CObject

    e = Elements()
    e.Drift(length=1.0)
    e.cbuffer.add_object(TYPE_TRICUB, np.zeros(3, np.uint64))
    assert isinstance(e.get(1), CObject)
    assert parameter_table(e, [])["begin"].size == 3


# ------------------------------------------- the reference's shipped lines
class _LineElement:
    """A pysixtrack element as the shipped line holds it: its class name and
    attributes, with to_dict(keepextra=True)."""

    def __init__(self, cls_name, attrs):
        self.__class__ = type(cls_name, (_LineElement,), {})
        self._attrs = attrs

    def to_dict(self, keepextra=False):
        return dict(self._attrs)


BB4D_KEYS = ("q_part", "N_part", "sigma_x", "sigma_y", "beta_s", "min_sigma_diff", "Delta_x",
             "Delta_y", "Dpx_sub", "Dpy_sub", "enabled")


@pytest.mark.parametrize("name,image", [("bbsimple", "bbsimple.npz"),
                                        ("beambeam", "ref_shipped_beambeam.npz")])
def test_shipped_line_converts_to_the_shipped_lattice(name, image):
    """The pysixtrack lines of the reference's `bbsimple` and `beambeam` test
    data (tests/golden/line_<name>.json.gz) converted here reproduce the
    lattices the reference wrote from them (beam_elements.bin, via
    Elements.fromline, python/sixtracklib/beam_elements.py:748-757): same
    element types in the same order, Drift / Multipole / Cavity words
    identical, the beam-beam payloads within 4e-16.  The line predates the
    named beam-beam parameters: its BeamBeam4D lists the payload in order
    (BB4D_data, be_beamfields.h:36-56), its BeamBeam6D the lab-frame strong
    beam that beam_elements.bb6d_data and gaussian_equal_charge_slices set
    up."""
    import gzip
    import json
    import os

    from sixtracklib_gb300 import CBuffer
    from sixtracklib_gb300.beam_elements import gaussian_equal_charge_slices

    golden = os.path.join(os.path.dirname(__file__), "golden")
    with gzip.open(os.path.join(golden, f"line_{name}.json.gz"), "rt") as f:
        items = json.load(f)
    beam_beam = []
    e = Elements()
    for cls_name, attrs in items:
        if cls_name in ("Drift", "Multipole", "Cavity"):
            e.append_line(SimpleNamespace(elements=[_LineElement(cls_name, attrs)]))
        elif cls_name == "BeamBeam4D":
            e.BeamBeam4D(data=[float(attrs[k]) for k in BB4D_KEYS])
            beam_beam.append(len(e) - 1)
        else:
            assert cls_name == "BeamBeam6D"
            charge, z = gaussian_equal_charge_slices(attrs["N_part_tot"], attrs["sigmaz"],
                                                     int(attrs["N_slices"]))
            sig = [attrs[f"Sig_{ij}_0"] for ij in ("11", "12", "13", "14", "22", "23", "24",
                                                   "33", "34", "44")]
            e.BeamBeam6D(data=bb6d_data(
                q_part=attrs["q_part"], phi=attrs["phi"], alpha=attrs["alpha"],
                delta_x=attrs["delta_x"], delta_y=attrs["delta_y"], n_part_per_slice=charge,
                z_slices=z, sigmas=sig,
                co=[attrs[k] for k in ("x_CO", "px_CO", "y_CO", "py_CO", "sigma_CO",
                                       "delta_CO")],
                min_sigma_diff=attrs["min_sigma_diff"],
                threshold_singular=attrs["threshold_singular"],
                d_sub=[attrs[k] for k in ("Dx_sub", "Dpx_sub", "Dy_sub", "Dpy_sub", "Dsigma_sub",
                                          "Ddelta_sub")],
                enabled=float(attrs["enabled"])))
            beam_beam.append(len(e) - 1)
    ref = Elements(cbuffer=CBuffer.from_image(np.load(os.path.join(golden, image))["lattice"]))
    mine, theirs = e.cbuffer.objects, ref.cbuffer.objects
    assert len(mine) == len(theirs) == len(items)
    for k, (a, b) in enumerate(zip(mine, theirs)):
        assert a.typeid == b.typeid, k
        if k in beam_beam:
            da = np.asarray(e.get(k).data, dtype=np.float64)
            db = np.asarray(ref.get(k).data, dtype=np.float64)
            assert da.shape == db.shape, k
            wa, wb = da.view(np.uint64), db.view(np.uint64)
            if a.typeid == 9:  # BeamBeam6D: slice count and relative offsets are integers
                assert wa[18] == wb[18] and np.array_equal(wa[34:38], wb[34:38])
                real = np.r_[0:18, 19:33, 38:da.size]
                assert (da[33] > 0) == (db[33] > 0)  # `enabled`: integer 1 there, 1.0 here
            else:
                real = np.r_[0:10]
                assert (da[10] > 0) == (db[10] > 0)
            dev = np.abs(da[real] - db[real])
            assert np.all((dev == 0) | (dev <= 4e-16 * np.abs(db[real]))), k
        else:  # every field of the element, arrays (the multipole's bal) included
            ea, eb = e.get(k), ref.get(k)
            for field, _ in type(ea)._fields:
                assert np.array_equal(np.asarray(getattr(ea, field)),
                                      np.asarray(getattr(eb, field))), (k, field)
