"""Element conversion to and from pysixtrack (python/sixtracklib/
pysixtrack_helper.py:1-141).

``BeamElementConverter`` maps the engine's element types onto pysixtrack's
by type id: Drift (2), DriftExact (3), Multipole (4), Cavity (5), XYShift
(6), SRotation (7), BeamBeam4D (8), BeamMonitor (10); the reference leaves
BeamBeam6D out of this map, and so does this one.  ``from_pysixtrack``
builds an engine element from any object with ``as_dict()`` whose class
name is one of those types; ``to_pysixtrack`` needs pysixtrack itself and
raises ImportError without it.
"""

from __future__ import annotations

import importlib.util

from .beam_elements import (BeamBeam4D, BeamMonitor, Cavity, Drift, DriftExact, Multipole,
                            SRotation, XYShift)


class BeamElementConverter:
    _type_id_to_elem_map = {2: Drift, 3: DriftExact, 4: Multipole, 5: Cavity, 6: XYShift,
                            7: SRotation, 8: BeamBeam4D, 10: BeamMonitor}
    _pysixtrack_to_type_id_map = {"Drift": 2, "DriftExact": 3, "Multipole": 4, "Cavity": 5,
                                  "XYShift": 6, "SRotation": 7, "BeamBeam4D": 8,
                                  "BeamMonitor": 10}

    @staticmethod
    def get_elemtype(type_id):
        """The engine element class of a type id, or None."""
        return BeamElementConverter._type_id_to_elem_map.get(type_id, None)

    @classmethod
    def get_typeid(cls):
        """The type id of the element class ``cls``, or None."""
        inv = {v: k for k, v in BeamElementConverter._type_id_to_elem_map.items()}
        return inv.get(cls, None)

    @staticmethod
    def available() -> bool:
        """True when pysixtrack can be imported (needed by to_pysixtrack)."""
        return importlib.util.find_spec("pysixtrack") is not None

    @staticmethod
    def to_pysixtrack(elem):
        """The pysixtrack element for an engine element, or None for types
        outside the map."""
        if not BeamElementConverter.available():
            raise ImportError("to_pysixtrack needs the pysixtrack package")
        from pysixtrack import elements as px

        type_id = getattr(elem, "_typeid", None)
        if BeamElementConverter.get_elemtype(type_id) is None:
            return None
        if type_id == 2:
            return px.Drift(length=elem.length)
        if type_id == 3:
            return px.DriftExact(length=elem.length)
        if type_id == 4:
            return px.Multipole(knl=elem.knl, ksl=elem.ksl, hxl=elem.hxl, hyl=elem.hyl,
                                length=elem.length)
        if type_id == 5:
            return px.Cavity(voltage=elem.voltage, frequency=elem.frequency, lag=elem.lag)
        if type_id == 6:
            return px.XYShift(dx=elem.dx, dy=elem.dy)
        if type_id == 7:
            return px.SRotation(angle=elem.angle_deg)
        if type_id == 8:
            d = [float(v) for v in elem.data]
            names = ("q_part", "N_part", "sigma_x", "sigma_y", "beta_s", "min_sigma_diff",
                     "Delta_x", "Delta_y", "Dpx_sub", "Dpy_sub", "enabled")
            return px.BeamBeam4D(**dict(zip(names, d)))
        return px.BeamMonitor(num_stores=elem.num_stores, start=elem.start, skip=elem.skip,
                              max_particle_id=elem.max_particle_id,
                              min_particle_id=elem.min_particle_id,
                              is_rolling=elem.is_rolling, is_turn_ordered=elem.is_turn_ordered)

    @staticmethod
    def from_pysixtrack(elem, cbuffer=None):
        """The engine element for a pysixtrack element (appended to
        ``cbuffer`` if given), or None for types outside the map."""
        type_id = BeamElementConverter._pysixtrack_to_type_id_map.get(
            elem.__class__.__name__)
        if type_id is None:
            return None
        return BeamElementConverter._type_id_to_elem_map[type_id](cbuffer=cbuffer,
                                                                  **elem.as_dict())
