"""MAD-X sequence conversion (python/sixtracklib/mad_helper.py:1-57).

A thin MAD-X sequence (every element of zero length, as MAD-X's
``makethin`` leaves it; cpymad's ``Sequence`` object or anything with the
same attributes) becomes a stream of ``(label, element class name,
parameters)``: a ``Drift`` for every gap between consecutive element
positions, then the element itself mapped onto the engine's element types
by its MAD-X base type.  ``Elements.from_mad`` builds a lattice from it.

Mapping (the reference's rules):

* ``multipole``: ``Multipole(knl, ksl, hxl=knl[0], hyl=0, length=lrad)``
  (a missing ``knl`` / ``ksl`` is ``[0]``);
* ``marker``, ``hmonitor``, ``vmonitor``, ``instrument``, ``monitor``,
  ``rcollimator``: a zero-length ``Drift``;
* ``hkicker``: ``Multipole(knl=[-kick], length=lrad)``; ``vkicker``:
  ``Multipole(ksl=[kick], length=lrad)``;
* ``rfcavity``: ``Cavity(voltage=volt * 1e6, frequency=freq * 1e6,
  lag=lag * 360)`` (MAD-X gives MV, MHz and the lag in units of 2 pi);
* any other base type is passed through unchanged, and building a lattice
  from it fails (``Elements`` has no such element).
"""

from __future__ import annotations

from collections import namedtuple

classes = dict(
    Drift=namedtuple("Drift", "length"),
    Multipole=namedtuple("Multipole", "knl ksl hxl hyl length"),
    Cavity=namedtuple("Cavity", "voltage frequency lag"),
    XYShift=namedtuple("XYShift", "dx dy"),
    SRotation=namedtuple("SRotation", "angle"),
    Line=namedtuple("Line", "elems"),
)

_AS_MARKER = ("marker", "hmonitor", "vmonitor", "instrument", "monitor", "rcollimator")


def dispatch(el, classes=classes):
    """The engine element for one thin MAD-X element (module doc)."""
    kind = el.base_type.name
    if kind == "multipole":
        knl = el.knl if hasattr(el, "knl") else [0]
        ksl = el.ksl if hasattr(el, "ksl") else [0]
        return classes["Multipole"](knl=knl, ksl=ksl, hxl=knl[0], hyl=0, length=el.lrad)
    if kind in _AS_MARKER:
        return classes["Drift"](length=0)
    if kind == "hkicker":
        return classes["Multipole"](knl=[-el.kick], ksl=[], hxl=0, hyl=0, length=el.lrad)
    if kind == "vkicker":
        return classes["Multipole"](knl=[], ksl=[el.kick], hxl=0, hyl=0, length=el.lrad)
    if kind == "rfcavity":
        return classes["Cavity"](voltage=el.volt * 1e6, frequency=el.freq * 1e6,
                                 lag=el.lag * 360)
    return el


def madseq_to_generator(seq, convert=classes):
    """``(label, class name, element)`` for a thin sequence: a ``Drift``
    (label ``"drift"``) for each positive gap between element positions,
    then the element.  Raises ValueError for an element of non-zero
    length."""
    drift = convert["Drift"]
    previous = 0
    for name, pos, el in zip(seq.element_names(), seq.element_positions(), seq.elements):
        if el.length > 0:
            raise ValueError(f"sequence {seq} contains {el} with length > 0")
        gap = pos - previous
        if gap > 0:
            yield "drift", "Drift", drift(gap)
        el = dispatch(el, convert)
        previous = pos
        yield name, el.__class__.__name__, el
