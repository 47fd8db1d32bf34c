"""Beam-element classes that encode into / decode from CObjects buffers.

Class names, constructor arguments and stored layouts follow the reference's
Python layer (python/sixtracklib/beam_elements.py:42-700) and C structs
(sixtracklib/common/be_*/be_*.h); the type ids are those of
sixtracklib/common/internal/objects_type_id.h:16-55.  Unlike the reference,
these classes need no ``cobjects`` package: they write the buffer through
:mod:`sixtracklib_gb300.cbuffer`.
"""

from __future__ import annotations

from math import factorial

import numpy as np

from .cbuffer import CBuffer, CObject

QELEM = 1.60217662e-19  # sixtracklib/common/constants.h:35
# q_part of beam-beam elements built from named parameters: the reference's
# Python binding uses scipy.constants.e there (beam_elements.py:11, :490, :508)
Q_PART_NAMED = 1.602176634e-19

TYPE_DRIFT = 2
TYPE_DRIFT_EXACT = 3
TYPE_MULTIPOLE = 4
TYPE_CAVITY = 5
TYPE_XYSHIFT = 6
TYPE_SROTATION = 7
TYPE_BEAM_BEAM_4D = 8
TYPE_BEAM_BEAM_6D = 9
TYPE_BEAM_MONITOR = 10
TYPE_LIMIT_RECT = 11
TYPE_LIMIT_ELLIPSE = 12
TYPE_SC_COASTING = 13
TYPE_SC_QGAUSSIAN_PROF = 14
TYPE_LIMIT_RECT_ELLIPSE = 16
TYPE_DIPEDGE = 24
TYPE_RF_MULTIPOLE = 256
TYPE_SC_INTERPOLATED_PROF = 257
TYPE_LINE_DENSITY_PROF_DATA = 258
TYPE_TRICUB_DATA = 260
TYPE_TRICUB = 261
TYPE_PARTICLE = 1


class _Element:
    """Base: ``_fields`` lists ``(name, kind)`` with kind 'f' (float64),
    'i' (int64), 'u' (uint64) or ('p', length_expr) for a pointer to a
    float64 array whose length is computed from the other fields."""

    _typeid = 0
    _fields: tuple = ()

    def __init__(self, cbuffer=None, **kwargs):
        for name, kind in self._fields:
            default = 0.0 if kind == "f" else 0
            if isinstance(kind, tuple):
                default = None
            setattr(self, name, kwargs.pop(name, getattr(self, "_default_" + name, default)))
        self._index = None
        self._cbuffer = None
        if cbuffer is not None:
            self._index = cbuffer.add_object(*self._encode())
            self._cbuffer = cbuffer
            cbuffer.typeids.setdefault(self._typeid, type(self))

    def _encode(self):
        words = np.zeros(len(self._fields), dtype=np.uint64)
        arrays = []
        for i, (name, kind) in enumerate(self._fields):
            v = getattr(self, name)
            if kind == "f":
                words[i] = np.float64(v).view(np.uint64)
            elif kind == "i":
                words[i] = np.int64(v).view(np.uint64)
            elif kind == "u":
                words[i] = np.uint64(int(v))
            else:
                arr = np.asarray(v if v is not None else [], dtype=np.float64)
                arrays.append((i, arr))
        return self._typeid, words, arrays

    @classmethod
    def _from_cobject(cls, obj: CObject, cbuffer=None, index=None):
        w = obj.words
        if w.size < len(cls._fields):  # truncated object: left undecoded
            return obj
        self = cls.__new__(cls)
        for i, (name, kind) in enumerate(cls._fields):
            if kind == "f":
                setattr(self, name, float(w[i : i + 1].view(np.float64)[0]))
            elif kind == "i":
                setattr(self, name, int(w[i : i + 1].view(np.int64)[0]))
            elif kind == "u":
                setattr(self, name, int(w[i]))
            else:
                off = int(w[i])
                n = cls._array_len(self, kind[1])
                setattr(self, name, w[off : off + n].view(np.float64).copy())
        self._index = index
        self._cbuffer = cbuffer
        return self

    @staticmethod
    def _array_len(self, expr):
        return int(eval(expr, {}, dict(self.__dict__)))

    def __setattr__(self, name, value):
        """Fields of an element that belongs to a lattice buffer are views of
        it, as the reference's CObject fields are: assigning one writes the
        buffer in place (an array field keeps its length)."""
        object.__setattr__(self, name, value)
        cb = self.__dict__.get("_cbuffer")
        index = self.__dict__.get("_index")
        if cb is None or index is None:
            return
        for fi, (fname, kind) in enumerate(self._fields):
            if fname == name:
                break
        else:
            return
        obj = cb.objects[index]
        if kind == "f":
            obj.words[fi] = np.float64(value).view(np.uint64)
        elif kind == "i":
            obj.words[fi] = np.int64(value).view(np.uint64)
        elif kind == "u":
            obj.words[fi] = np.uint64(int(value))
        else:
            arr = np.ascontiguousarray(value, dtype=np.float64).ravel()
            off = int(obj.words[fi])
            n = self._array_len(self, kind[1])
            if arr.size != n:
                raise ValueError(f"{type(self).__name__}.{name}: {arr.size} values for an "
                                 f"array of {n} in the buffer (its layout is fixed)")
            obj.words[off:off + n] = arr.view(np.uint64)
            object.__setattr__(self, name, arr.copy())
        cb.touch()

    def _set_array_entry(self, name, i, value):
        """array field ``name``[i] = value, here and in the lattice buffer
        the element belongs to (the reference's elements are views of their
        buffer, so its setters write the buffer in place)."""
        getattr(self, name)[i] = value
        if self._cbuffer is not None and self._index is not None:
            fi = [f for f, _ in self._fields].index(name)
            obj = self._cbuffer.objects[self._index]
            obj.words[int(obj.words[fi]) + i] = np.float64(value).view(np.uint64)
            self._cbuffer.touch()

    def to_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields}

    def __repr__(self):
        args = ", ".join(f"{k}={v!r}" for k, v in self.to_dict().items())
        return f"{type(self).__name__}({args})"


class Drift(_Element):
    _typeid = TYPE_DRIFT
    _fields = (("length", "f"),)


class DriftExact(_Element):
    _typeid = TYPE_DRIFT_EXACT
    _fields = (("length", "f"),)


def _knl_ksl_to_bal(order, knl, ksl):
    knl = [] if knl is None else list(knl)
    ksl = [] if ksl is None else list(ksl)
    order = 0 if order is None else int(order)
    n = max(order + 1, len(knl), len(ksl))
    kn = np.zeros(n)
    ks = np.zeros(n)
    kn[: len(knl)] = knl
    ks[: len(ksl)] = ksl
    inv_fact = np.array([1.0 / factorial(i) for i in range(n)])
    bal = np.zeros(2 * n)
    bal[0::2] = kn * inv_fact
    bal[1::2] = ks * inv_fact
    return n - 1, bal


class _BalAccess:
    """knl / ksl of ``bal`` (bal[2k] = knl[k] / k!, bal[2k+1] = ksl[k] / k!)
    and their in-place setters (python/sixtracklib/beam_elements.py:112-128,
    :232-248)."""

    @property
    def knl(self):
        return np.array([self.bal[2 * k] * factorial(k) for k in range(self.order + 1)])

    @property
    def ksl(self):
        return np.array([self.bal[2 * k + 1] * factorial(k) for k in range(self.order + 1)])

    def set_knl(self, value, order):
        assert order <= self.order
        self._set_array_entry("bal", 2 * order, float(np.squeeze(value)) / factorial(order))

    def set_ksl(self, value, order):
        assert order <= self.order
        self._set_array_entry("bal", 2 * order + 1, float(np.squeeze(value)) / factorial(order))


class Multipole(_BalAccess, _Element):
    """Thin multipole; ``bal[2k] = knl[k]/k!``, ``bal[2k+1] = ksl[k]/k!``
    (be_multipole.h:449-466)."""

    _typeid = TYPE_MULTIPOLE
    _fields = (
        ("order", "i"),
        ("length", "f"),
        ("hxl", "f"),
        ("hyl", "f"),
        ("bal", ("p", "2*order+2")),
    )

    def __init__(self, order=None, knl=None, ksl=None, bal=None, cbuffer=None, **kw):
        if bal is None:
            order, bal = _knl_ksl_to_bal(order, knl, ksl)
        else:
            bal = np.asarray(bal, dtype=np.float64)
            order = (len(bal) - 2) // 2
        super().__init__(cbuffer=cbuffer, order=order, bal=bal, **kw)


class RFMultipole(_BalAccess, _Element):
    _typeid = TYPE_RF_MULTIPOLE
    _fields = (
        ("order", "i"),
        ("voltage", "f"),
        ("frequency", "f"),
        ("lag", "f"),
        ("bal", ("p", "2*order+2")),
        ("phase", ("p", "2*order+2")),
    )

    def __init__(self, order=None, knl=None, ksl=None, pn=None, ps=None, bal=None,
                 p=None, cbuffer=None, **kw):
        if bal is None:
            knl, ksl, pn, ps = ([] if a is None else list(np.atleast_1d(a))
                                for a in (knl, ksl, pn, ps))
            n = max([(order or 0) + 1] + [len(a) for a in (knl, ksl, pn, ps)])
            order, bal = _knl_ksl_to_bal(n - 1, knl, ksl)
            ph = np.zeros(2 * n)
            ph[0::2][: len(pn)] = pn
            ph[1::2][: len(ps)] = ps
        else:
            bal = np.asarray(bal, dtype=np.float64)
            ph = np.asarray(p if p is not None else kw.pop("phase"), dtype=np.float64)
            order = (len(bal) - 2) // 2
        kw.pop("phase", None)
        super().__init__(cbuffer=cbuffer, order=order, bal=bal, phase=ph, **kw)

    @property
    def pn(self):
        return np.asarray(self.phase)[0::2].copy()

    @property
    def ps(self):
        return np.asarray(self.phase)[1::2].copy()

    def set_pn(self, value, order):
        assert order <= self.order
        self._set_array_entry("phase", 2 * order, float(np.squeeze(value)))

    def set_ps(self, value, order):
        assert order <= self.order
        self._set_array_entry("phase", 2 * order + 1, float(np.squeeze(value)))


class Cavity(_Element):
    _typeid = TYPE_CAVITY
    _fields = (("voltage", "f"), ("frequency", "f"), ("lag", "f"))


class XYShift(_Element):
    _typeid = TYPE_XYSHIFT
    _fields = (("dx", "f"), ("dy", "f"))


class SRotation(_Element):
    """Rotation about s; ``angle`` in degrees (beam_elements.py:282-300)."""

    _typeid = TYPE_SROTATION
    _fields = (("cos_z", "f"), ("sin_z", "f"))
    _default_cos_z = 1.0

    def __init__(self, angle=None, cbuffer=None, **kw):
        if angle is not None:
            a = angle / 180 * np.pi
            kw["cos_z"] = float(np.cos(a))
            kw["sin_z"] = float(np.sin(a))
        super().__init__(cbuffer=cbuffer, **kw)

    @property
    def angle(self):
        """The rotation angle in radians (beam_elements.py:293-295; the
        constructor takes degrees)."""
        return float(np.arctan2(self.sin_z, self.cos_z))

    @property
    def angle_deg(self):
        return float(np.arctan2(self.sin_z, self.cos_z) * 180.0 / np.pi)


class BeamMonitor(_Element):
    _typeid = TYPE_BEAM_MONITOR
    _fields = (
        ("num_stores", "i"),
        ("start", "i"),
        ("skip", "i"),
        ("out_address", "u"),
        ("max_particle_id", "i"),
        ("min_particle_id", "i"),
        ("is_rolling", "i"),
        ("is_turn_ordered", "i"),
    )
    _default_skip = 1
    _default_is_turn_ordered = 1


def append_beam_monitors_to_lattice(beam_elements_buffer, until_turn_elem_by_elem,
                                    until_turn_turn_by_turn, until_turn, skip_turns=1,
                                    min_particle_id=0, max_particle_id=0, initial_at_turn=0):
    """Append the turn-by-turn and the periodic output monitors
    (beam_elements.py:314-367): a turn-ordered monitor storing every turn
    from max(initial_at_turn, until_turn_elem_by_elem) up to
    until_turn_turn_by_turn, then a rolling one storing every `skip_turns`-th
    turn up to until_turn.  Returns the number of monitors added."""
    cb = beam_elements_buffer
    if not isinstance(cb, CBuffer):
        cb = getattr(cb, "cbuffer", cb)
    added = 0
    start_tbt = max(initial_at_turn, until_turn_elem_by_elem)
    if until_turn_turn_by_turn > start_tbt:
        BeamMonitor(start=start_tbt, num_stores=until_turn_turn_by_turn - start_tbt, skip=1,
                    out_address=0, min_particle_id=min_particle_id,
                    max_particle_id=max_particle_id, is_rolling=0, is_turn_ordered=1,
                    cbuffer=cb)
        added += 1
    start_out = max(start_tbt, until_turn_turn_by_turn)
    if until_turn > start_out:
        skip = skip_turns if skip_turns > 0 else 1
        num_stores, rem = divmod(until_turn - start_out, skip)
        if rem > 0:
            num_stores += 1
        BeamMonitor(start=start_out, num_stores=num_stores, skip=skip, out_address=0,
                    min_particle_id=min_particle_id, max_particle_id=max_particle_id,
                    is_rolling=1, is_turn_ordered=1, cbuffer=cb)
        added += 1
    return added


class LimitRect(_Element):
    _typeid = TYPE_LIMIT_RECT
    _fields = (("min_x", "f"), ("max_x", "f"), ("min_y", "f"), ("max_y", "f"))

    def __init__(self, min_x=None, max_x=None, min_y=None, max_y=None,
                 min_coord=-1.0, max_coord=1.0, cbuffer=None, **kw):
        min_x = min_coord if min_x is None else min_x
        min_y = min_coord if min_y is None else min_y
        max_x = max_coord if max_x is None else max_x
        max_y = max_coord if max_y is None else max_y
        if min_x > max_x:
            min_x, max_x = max_x, min_x
        if min_y > max_y:
            min_y, max_y = max_y, min_y
        if (max_x - min_x) * (max_y - min_y) <= 0.0:
            raise ValueError("min_x, max_x, min_y, max_y have to delimit a non-vanishing rectangle")
        super().__init__(cbuffer=cbuffer, min_x=min_x, max_x=max_x, min_y=min_y, max_y=max_y, **kw)


class LimitEllipse(_Element):
    _typeid = TYPE_LIMIT_ELLIPSE
    _fields = (("a_squ", "f"), ("b_squ", "f"), ("a_b_squ", "f"))

    def __init__(self, a_squ=None, b_squ=None, a=None, b=None, cbuffer=None, **kw):
        if a_squ is None:
            a_squ = a * a if (a is not None and a > 0.0) else 1.0
        if b_squ is None:
            b_squ = b * b if (b is not None and b > 0.0) else 1.0
        if not (a_squ > 0.0 and b_squ > 0.0):
            raise ValueError("a_squ and b_squ have to be positive definite")
        kw.pop("a_b_squ", None)
        super().__init__(cbuffer=cbuffer, a_squ=a_squ, b_squ=b_squ, a_b_squ=a_squ * b_squ, **kw)

    def set_half_axes(self, a, b):
        return self.set_half_axes_squ(a * a, b * b)

    def set_half_axes_squ(self, a_squ, b_squ):
        """beam_elements.py:460-467 / 647-654 (written into the lattice
        buffer the element belongs to)."""
        self.a_squ = a_squ
        self.b_squ = b_squ
        self.a_b_squ = a_squ * b_squ
        return self


class LimitRectEllipse(_Element):
    _typeid = TYPE_LIMIT_RECT_ELLIPSE
    _fields = (("max_x", "f"), ("max_y", "f"), ("a_squ", "f"), ("b_squ", "f"), ("a_b_squ", "f"))

    def __init__(self, max_x=1.0, max_y=1.0, a_squ=None, b_squ=None, a=None, b=None,
                 cbuffer=None, **kw):
        if a_squ is None:
            a_squ = a * a if (a is not None and a > 0.0) else 1.0
        if b_squ is None:
            b_squ = b * b if (b is not None and b > 0.0) else 1.0
        if max_x < 0.0 or max_y < 0.0 or a_squ < 0.0 or b_squ < 0.0:
            raise ValueError("LimitRectEllipse parameters have to be positive definite")
        kw.pop("a_b_squ", None)
        super().__init__(cbuffer=cbuffer, max_x=max_x, max_y=max_y, a_squ=a_squ,
                         b_squ=b_squ, a_b_squ=a_squ * b_squ, **kw)

    def set_half_axes(self, a, b):
        return self.set_half_axes_squ(a * a, b * b)

    def set_half_axes_squ(self, a_squ, b_squ):
        """beam_elements.py:460-467 / 647-654 (written into the lattice
        buffer the element belongs to)."""
        self.a_squ = a_squ
        self.b_squ = b_squ
        self.a_b_squ = a_squ * b_squ
        return self


class DipoleEdge(_Element):
    _typeid = TYPE_DIPEDGE
    _fields = (("r21", "f"), ("r43", "f"))

    def __init__(self, r21=None, r43=None, h=0.0, e1=0.0, hgap=0.0, fint=0.0,
                 cbuffer=None, **kw):
        if r21 is None and r43 is None:
            corr = 2.0 * h * hgap * fint
            r21 = h * np.tan(e1)
            temp = corr / np.cos(e1) * (1.0 + np.sin(e1) * np.sin(e1))
            r43 = -h * np.tan(e1 - temp)
        super().__init__(cbuffer=cbuffer, r21=float(r21), r43=float(r43), **kw)


class _DataElement(_Element):
    """{size, data_addr} elements whose payload is a float64 array."""

    _fields = (("size", "u"), ("data", ("p", "size")))

    def __init__(self, data=None, cbuffer=None, **kw):
        data = np.asarray(data if data is not None else [], dtype=np.float64)
        kw.pop("size", None)
        super().__init__(cbuffer=cbuffer, size=data.size, data=data, **kw)


class BeamBeam4D(_DataElement):
    """4D weak-strong beam-beam; payload = [q_part, N_part, sigma_x, sigma_y,
    beta_s, min_sigma_diff, Delta_x, Delta_y, Dpx_sub, Dpy_sub, enabled]
    (be_beamfields.h:36-56, beam_elements.py:470-494)."""

    _typeid = TYPE_BEAM_BEAM_4D

    def __init__(self, data=None, cbuffer=None, **kw):
        if data is None and "x_bb" in kw:
            keys = ("charge", "sigma_x", "sigma_y", "beta_r", "min_sigma_diff",
                    "x_bb", "y_bb", "d_px", "d_py", "enabled")
            data = [Q_PART_NAMED] + [float(kw.pop(k)) for k in keys]
        super().__init__(data=data, cbuffer=cbuffer, **kw)


class BeamBeam6D(_DataElement):
    """6D synchro-beam; payload = the BB6D data block
    (be_beamfields.h:222-250), see :func:`bb6d_data`.

    Like the reference (beam_elements.py:496-543) it also takes the strong
    beam's parameters by name, as a pysixtrack ``BeamBeam6D`` lists them --
    ``phi``, ``alpha``, ``x_bb_co``, ``y_bb_co``, ``charge_slices``,
    ``zeta_slices``, ``sigma_11`` .. ``sigma_44``, ``x_co`` .. ``delta_co``,
    ``min_sigma_diff``, ``threshold_singular``, ``d_x`` .. ``d_delta``,
    ``enabled`` -- and builds the payload with :func:`bb6d_data` (the
    reference calls pysixtrack's initialisation there)."""

    _typeid = TYPE_BEAM_BEAM_6D

    def __init__(self, data=None, cbuffer=None, **kw):
        if data is None and "x_bb_co" in kw:
            sig = [kw[f"sigma_{ij}"] for ij in ("11", "12", "13", "14", "22", "23", "24",
                                                "33", "34", "44")]
            data = bb6d_data(
                q_part=Q_PART_NAMED, phi=kw["phi"], alpha=kw["alpha"], delta_x=kw["x_bb_co"],
                delta_y=kw["y_bb_co"], n_part_per_slice=kw["charge_slices"],
                z_slices=kw["zeta_slices"], sigmas=sig,
                co=[kw[k] for k in ("x_co", "px_co", "y_co", "py_co", "zeta_co", "delta_co")],
                min_sigma_diff=kw["min_sigma_diff"],
                threshold_singular=kw["threshold_singular"],
                d_sub=[kw[k] for k in ("d_x", "d_px", "d_y", "d_py", "d_zeta", "d_delta")],
                enabled=kw["enabled"])
        super().__init__(data=data, cbuffer=cbuffer, **kw)


class SCCoasting(_Element):
    _typeid = TYPE_SC_COASTING
    _fields = (
        ("number_of_particles", "f"),
        ("circumference", "f"),
        ("sigma_x", "f"),
        ("sigma_y", "f"),
        ("length", "f"),
        ("x_co", "f"),
        ("y_co", "f"),
        ("min_sigma_diff", "f"),
        ("enabled", "u"),
    )
    _default_circumference = 1.0
    _default_sigma_x = 1.0
    _default_sigma_y = 1.0
    _default_min_sigma_diff = 1e-10
    _default_enabled = 1


class SCQGaussProfile(_Element):
    _typeid = TYPE_SC_QGAUSSIAN_PROF
    _fields = (
        ("number_of_particles", "f"),
        ("bunchlength_rms", "f"),
        ("sigma_x", "f"),
        ("sigma_y", "f"),
        ("length", "f"),
        ("x_co", "f"),
        ("y_co", "f"),
        ("min_sigma_diff", "f"),
        ("q_param", "f"),
        ("cq", "f"),
        ("enabled", "u"),
    )
    _default_bunchlength_rms = 1.0
    _default_sigma_x = 1.0
    _default_sigma_y = 1.0
    _default_min_sigma_diff = 1e-10
    _default_q_param = 1.0
    _default_cq = float(np.sqrt(np.pi))
    _default_enabled = 1

    def __init__(self, cbuffer=None, **kw):
        if "cq" not in kw:
            kw["cq"] = q_gauss_cq(kw.get("q_param", 1.0))
        super().__init__(cbuffer=cbuffer, **kw)


def q_gauss_cq(q):
    """Normalisation of the q-Gaussian (internal/math_qgauss.h:140-165)."""
    from math import gamma, sqrt, pi

    eps = 1e-6
    cq = sqrt(pi)
    if q >= 1.0 + eps:
        cq *= gamma((3.0 - q) / (2.0 * (q - 1.0)))
        cq /= sqrt(q - 1.0) * gamma(1.0 / (q - 1.0))
    elif q <= 1.0 - eps:
        cq *= 2.0 * gamma(1.0 / (1.0 - q))
        cq /= (3.0 - q) * sqrt(1.0 - q) * gamma((3.0 - q) / (2.0 * (1.0 - q)))
    return cq


def interpolation_derivatives(values, dz, method):
    """Derivative table of a line-density profile as the reference prepares
    it (NS(Math_interpol_prepare_equ), internal/math_interpol.h:604-645):
    linear -- forward slopes ``(y[i+1] - y[i]) / dz`` (last entry 0,
    :322-367); cubic -- second derivatives of the natural cubic spline
    (tridiagonal solve of :369-600 with natural boundaries)."""
    y = np.asarray(values, dtype=np.float64)
    n = y.size
    out = np.zeros(n)
    if method == 0:
        if n > 1:
            out[:-1] = (y[1:] - y[:-1]) / dz
        return out
    if method != 1:
        return out
    if n <= 3:
        raise ValueError("cubic interpolation needs more than 3 values")
    h = np.full(n, float(dz))
    g = np.zeros(n)
    d = np.zeros(n)
    l_ = np.zeros(n)
    dy = np.zeros(n)
    for i in range(1, n - 1):
        g[i] = (h[i - 1] + h[i]) * 2.0
        t = (y[i + 1] - y[i]) / h[i]
        t -= (y[i] - y[i - 1]) / h[i - 1]
        dy[i] = t * 6.0
    d[0] = g[1]
    out[0] = dy[1]
    for i in range(1, n - 2):
        l_[i] = h[i] / d[i - 1]
        d[i] = g[i + 1] - l_[i] * h[i]
        out[i] = dy[i + 1] - out[i - 1] * l_[i]
    i = n - 3
    out[i + 1] = out[i] / d[i]
    for i in range(n - 4, -1, -1):
        out[i + 1] = (out[i] - h[i + 1] * out[i + 2]) / d[i]
    out[0] = 0.0
    out[n - 1] = 0.0
    return out


class LineDensityProfileData(_Element):
    """Tabulated longitudinal line density (be_beamfields.h:887-897): values
    on the grid ``z0 + k dz`` and the derivative table for ``method`` 0
    (linear) or 1 (cubic); 255 disables interpolation.  The arrays have
    ``capacity`` entries, of which ``num_values`` are used."""

    _typeid = TYPE_LINE_DENSITY_PROF_DATA

    @staticmethod
    def ptr_offset():
        """Offset added to the object's address when it is assigned to an
        SCInterpolatedProfile (sc_line_density.py:72-74)."""
        return 0

    _fields = (
        ("method", "u"),
        ("capacity", "i"),
        ("values", ("p", "capacity")),
        ("derivatives", ("p", "capacity")),
        ("z0", "f"),
        ("dz", "f"),
        ("num_values", "i"),
    )
    METHODS = {"linear": 0, "cubic": 1, "none": 255}
    _default_dz = 1.0

    def __init__(self, values=None, z0=0.0, dz=1.0, method="linear", capacity=None,
                 derivatives=None, cbuffer=None, **kw):
        m = self.METHODS[method] if isinstance(method, str) else int(method)
        v = np.asarray(values if values is not None else [], dtype=np.float64)
        nv = v.size
        cap = max(int(capacity or 0), nv)
        vals = np.zeros(cap)
        vals[:nv] = v
        if derivatives is None:
            der = np.zeros(cap)
            der[:nv] = interpolation_derivatives(v, dz, m) if nv else []
        else:
            der = np.zeros(cap)
            der[: len(derivatives)] = derivatives
        kw.pop("num_values", None)
        super().__init__(cbuffer=cbuffer, method=m, capacity=cap, values=vals,
                         derivatives=der, z0=float(z0), dz=float(dz), num_values=nv, **kw)


class SCInterpolatedProfile(_Element):
    """Space-charge kick with a tabulated line density (be_beamfields.h:
    1281-1293).  ``line_density``: index of a :class:`LineDensityProfileData`
    object in the same buffer; its absolute address is written into
    ``interpol_data_addr`` whenever the buffer is serialised.  Without one
    (or with method 255 or no values) ``line_density_prof_fallback`` is the
    density, as in the reference."""

    _typeid = TYPE_SC_INTERPOLATED_PROF
    _fields = (
        ("number_of_particles", "f"),
        ("sigma_x", "f"),
        ("sigma_y", "f"),
        ("length", "f"),
        ("x_co", "f"),
        ("y_co", "f"),
        ("interpol_data_addr", "u"),
        ("line_density_prof_fallback", "f"),
        ("min_sigma_diff", "f"),
        ("enabled", "u"),
    )
    _default_sigma_x = 1.0
    _default_sigma_y = 1.0
    _default_line_density_prof_fallback = 1.0
    _default_min_sigma_diff = 1e-10
    _default_enabled = 1

    @staticmethod
    def interpol_data_addr_offset():
        """Byte offset of ``interpol_data_addr`` in the struct."""
        return 6 * 8

    def __init__(self, line_density=None, cbuffer=None, **kw):
        self.line_density = None if line_density is None else int(line_density)
        super().__init__(cbuffer=cbuffer, **kw)

    def _encode(self):
        typeid, words, arrays = super()._encode()
        links = [] if self.line_density is None else [(6, self.line_density)]
        return typeid, words, arrays, links

    @classmethod
    def _from_cobject(cls, obj: CObject, cbuffer=None, index=None):
        self = super()._from_cobject(obj, cbuffer, index)
        self.line_density = obj.links[0][1] if obj.links else None
        return self


# Aliases used by the reference's naming of the space-charge kicks.
SpaceChargeCoasting = SCCoasting
SpaceChargeQGaussianProfile = SCQGaussProfile
SpaceChargeBunched = SCQGaussProfile

class _BufferArray(np.ndarray):
    """float64 view of an array field inside a lattice buffer: item writes
    go to the buffer (and invalidate its cached image), as the reference's
    CObject array fields are views of their buffer."""

    def __array_finalize__(self, obj):
        self._cb = getattr(obj, "_cb", None)

    def __setitem__(self, key, value):
        super().__setitem__(key, value)
        if self._cb is not None:
            self._cb.touch()


class TriCubData(_Element):
    """Tricubic interpolation table (python/sixtracklib/tricub.py:21-49):
    grid origin, step and size per axis, mirror flags, and nx ny nz x 8
    values: f, df/dx, df/dy, df/dz, d2f/dxdy, d2f/dxdz, d2f/dydz,
    d3f/dxdydz (derivatives scaled by the grid steps) at node
    l + 8 (ix + nx (iy + ny iz)).  The table is zero-filled unless given;
    ``table_addr`` of an element in a buffer is a view of the buffer, so
    ``table_addr[i] = v`` edits the buffer, as with the reference.  The
    TriCub map is disabled in the reference's default build and here
    (a TriCubData in the lattice then fails to track too); the
    ``track_tricub`` configuration key enables or skips it."""

    _typeid = TYPE_TRICUB_DATA
    _fields = (
        ("x0", "f"), ("dx", "f"), ("nx", "i"),
        ("y0", "f"), ("dy", "f"), ("ny", "i"),
        ("z0", "f"), ("dz", "f"), ("nz", "i"),
        ("mirror_x", "i"), ("mirror_y", "i"), ("mirror_z", "i"),
        ("table_addr", ("p", "nx*ny*nz*8")),
    )

    def __init__(self, cbuffer=None, nx=0, ny=0, nz=0, table_addr=None, **kw):
        n = int(nx) * int(ny) * int(nz) * 8
        table = np.zeros(n) if table_addr is None else np.asarray(table_addr, dtype=np.float64)
        if table.size != n:
            raise ValueError(f"TriCubData: {table.size} table values for {n} = nx ny nz 8")
        super().__init__(cbuffer=cbuffer, nx=nx, ny=ny, nz=nz, table_addr=table.ravel(), **kw)
        self._attach_table()

    def _attach_table(self):
        cb, index = self.__dict__.get("_cbuffer"), self.__dict__.get("_index")
        if cb is None or index is None:
            return
        obj = cb.objects[index]
        off = int(obj.words[12])
        n = self._array_len(self, "nx*ny*nz*8")
        view = obj.words[off:off + n].view(np.float64).view(_BufferArray)
        view._cb = cb
        object.__setattr__(self, "table_addr", view)

    @classmethod
    def _from_cobject(cls, obj, cbuffer=None, index=None):
        self = super()._from_cobject(obj, cbuffer, index)
        if isinstance(self, cls):
            self._attach_table()
        return self

    def __setattr__(self, name, value):
        super().__setattr__(name, value)
        if name == "table_addr":
            self._attach_table()

    @staticmethod
    def ptr_offset():
        return 0


class TriCub(_Element):
    """Tricubic-interpolated kick element (python/sixtracklib/tricub.py:52-68);
    ``data_addr`` holds the address of its TriCubData: a job assigns it from
    a stored buffer (tricub.TriCub_buffer_create_assign_address_item), or
    ``data`` names a TriCubData of the same buffer, whose absolute address
    is written into ``data_addr`` whenever the buffer is serialised.  The map
    is disabled in the reference's default build and here (tracking through
    it fails); the ``track_tricub`` configuration key ("enabled", "skip",
    "disabled") selects it."""

    _typeid = TYPE_TRICUB
    _fields = (
        ("x_shift", "f"), ("y_shift", "f"), ("tau_shift", "f"),
        ("dipolar_kick_px", "f"), ("dipolar_kick_py", "f"), ("dipolar_kick_ptau", "f"),
        ("length", "f"), ("data_addr", "u"),
    )

    def __init__(self, data=None, cbuffer=None, **kw):
        self.data = None if data is None else int(data)
        super().__init__(cbuffer=cbuffer, **kw)

    def _encode(self):
        typeid, words, arrays = super()._encode()
        links = [] if self.data is None else [(7, self.data)]
        return typeid, words, arrays, links

    @classmethod
    def _from_cobject(cls, obj: CObject, cbuffer=None, index=None):
        self = super()._from_cobject(obj, cbuffer, index)
        if isinstance(self, cls):
            self.data = obj.links[0][1] if obj.links else None
        return self

    @staticmethod
    def data_addr_offset():
        return 7 * 8


ELEMENT_TYPES = {
    TYPE_DRIFT: Drift,
    TYPE_DRIFT_EXACT: DriftExact,
    TYPE_MULTIPOLE: Multipole,
    TYPE_RF_MULTIPOLE: RFMultipole,
    TYPE_CAVITY: Cavity,
    TYPE_XYSHIFT: XYShift,
    TYPE_SROTATION: SRotation,
    TYPE_BEAM_MONITOR: BeamMonitor,
    TYPE_LIMIT_RECT: LimitRect,
    TYPE_LIMIT_ELLIPSE: LimitEllipse,
    TYPE_LIMIT_RECT_ELLIPSE: LimitRectEllipse,
    TYPE_DIPEDGE: DipoleEdge,
    TYPE_BEAM_BEAM_4D: BeamBeam4D,
    TYPE_BEAM_BEAM_6D: BeamBeam6D,
    TYPE_SC_COASTING: SCCoasting,
    TYPE_SC_QGAUSSIAN_PROF: SCQGaussProfile,
    TYPE_SC_INTERPOLATED_PROF: SCInterpolatedProfile,
    TYPE_LINE_DENSITY_PROF_DATA: LineDensityProfileData,
    TYPE_TRICUB_DATA: TriCubData,
    TYPE_TRICUB: TriCub,
}


class Elements:
    """Lattice container (python/sixtracklib/beam_elements.py:705-800):
    ``Elements().Drift(length=1.0)`` appends a drift to ``self.cbuffer``."""

    element_types = {cls.__name__: cls for cls in ELEMENT_TYPES.values()}

    @staticmethod
    def add_element_type(cls, cls_name):
        """Register an element class under ``cls_name`` for Elements made
        from now on (beam_elements.py:732-734)."""
        Elements.element_types.update({cls_name: cls})

    def __init__(self, cbuffer=None):
        self.cbuffer = CBuffer() if cbuffer is None else cbuffer
        for tid, cls in ELEMENT_TYPES.items():
            self.cbuffer.typeids[tid] = cls
        for name, cls in self.element_types.items():
            setattr(self, name, self._mk(cls))
            self.cbuffer.typeids.setdefault(cls._typeid, cls)
        self._builder = self.gen_builder()

    def _mk(self, cls):
        def fun(*args, **kw):
            return cls(*args, cbuffer=self.cbuffer, **kw)

        return fun

    def gen_builder(self):
        """``{class name: function appending such an element}``."""
        return {name: getattr(self, name) for name in self.element_types}

    @classmethod
    def fromfile(cls, filename):
        return cls(cbuffer=CBuffer.fromfile(filename))

    @classmethod
    def from_line(cls, line):
        """A lattice from a pysixtrack-style line (beam_elements.py:748-757):
        ``line.elements``, each with ``to_dict(keepextra=True)``; the class
        name selects the element type."""
        return cls().append_line(line)

    def append_line(self, line):
        for element in line.elements:
            getattr(self, element.__class__.__name__)(**element.to_dict(keepextra=True))
        return self

    @classmethod
    def from_mad(cls, seq, exact_drift=False):
        """A lattice from a thin MAD-X sequence (beam_elements.py:786-795;
        conversion rules in :mod:`sixtracklib_gb300.mad_helper`);
        ``exact_drift`` makes the drifts DriftExact."""
        from .mad_helper import madseq_to_generator

        self = cls()
        for _label, name, element in madseq_to_generator(seq):
            if exact_drift and name == "Drift":
                name = "DriftExact"
            getattr(self, name)(**element._asdict())
        return self

    def to_file(self, filename):
        self.cbuffer.tofile(filename)
        return self

    def get_elements(self):
        return [self.cbuffer.get_object(i) for i in range(self.cbuffer.n_objects)]

    def get(self, i):
        return self.cbuffer.get_object(i)

    def __len__(self):
        return self.cbuffer.n_objects


def bb6d_data(q_part, phi, alpha, delta_x, delta_y, n_part_per_slice, z_slices,
              sigmas, co=(0, 0, 0, 0, 0, 0), min_sigma_diff=1e-10,
              threshold_singular=1e-28, d_sub=(0, 0, 0, 0, 0, 0), enabled=1.0):
    """Build a BeamBeam6D payload (layout be_beamfields.h:222-250).

    The reference delegates this initialisation to pysixtrack
    (``BB6Ddata.BB6D_init``, called at python/sixtracklib/beam_elements.py:
    496-543), which is not part of the reference tree.  This is an own
    implementation from the physics of the Hirata boost:

    * boost parameters: ``sin/cos/tan`` of the half crossing angle ``phi`` and
      ``sin/cos`` of the crossing-plane angle ``alpha``;
    * the boosted sigma matrix: the boost scales transverse momenta by
      ``1/cos(phi)``, so entries with one momentum index scale by
      ``1/cos(phi)`` and entries with two by ``1/cos(phi)**2``;
    * the strong-beam slice centroids (x=px=y=py=delta=0, sigma=z) are
      transformed with the same linear boost the tracking map applies to the
      weak beam: ``x* = cos(alpha) tan(phi) z``, ``y* = sin(alpha) tan(phi) z``,
      ``sigma* = z / cos(phi)``.

    ``sigmas`` = (S11, S12, S13, S14, S22, S23, S24, S33, S34, S44) in the lab
    frame; ``co`` = closed orbit (x, px, y, py, zeta, delta); ``d_sub`` =
    (Dx, Dpx, Dy, Dpy, Dzeta, Ddelta) dipolar subtraction.
    """
    sphi, cphi, tphi = np.sin(phi), np.cos(phi), np.tan(phi)
    salpha, calpha = np.sin(alpha), np.cos(alpha)
    z = np.asarray(z_slices, dtype=np.float64)
    n = z.size
    s11, s12, s13, s14, s22, s23, s24, s33, s34, s44 = [float(v) for v in sigmas]
    c2 = cphi * cphi
    sig_star = (s11, s12 / cphi, s13, s14 / cphi, s22 / c2, s23 / cphi,
                s24 / c2, s33, s34 / cphi, s44 / c2)
    head = [q_part, sphi, cphi, tphi, salpha, calpha, *sig_star,
            min_sigma_diff, threshold_singular, 0.0, delta_x, delta_y, *co,
            *d_sub, enabled]
    assert len(head) == 34
    words = np.zeros(38 + 4 * n, dtype=np.float64)
    words[:34] = head
    w = words.view(np.uint64)
    w[18] = np.uint64(n)
    for k, f in enumerate(range(34, 38)):
        w[f] = np.uint64(38 + k * n - f - 1)
    words[38 : 38 + n] = np.asarray(n_part_per_slice, dtype=np.float64)
    words[38 + n : 38 + 2 * n] = calpha * tphi * z
    words[38 + 2 * n : 38 + 3 * n] = salpha * tphi * z
    words[38 + 3 * n : 38 + 4 * n] = z / cphi
    return words


def gaussian_equal_charge_slices(n_part_tot, sigma_z, n_slices):
    """Slicing of a Gaussian strong bunch into `n_slices` slices of equal
    charge, as the 6D beam-beam set-up of the reference's Python layer
    expects them (charge_slices, zeta_slices): the bins are the quantiles
    k / n_slices of the longitudinal Gaussian, each slice sits at the
    centroid of its bin, sigma_z sqrt(n_slices^2 / (2 pi)) (exp(-a^2 / 2) -
    exp(-b^2 / 2)) for the normalised bin edges a < b, head (largest z)
    first; one slice sits at z = 0.  Returns (charge per slice, z)."""
    n = int(n_slices)
    if n < 1:
        raise ValueError("at least one slice")
    if n == 1:
        return np.array([float(n_part_tot)]), np.array([0.0])
    from scipy.special import ndtri

    edges = ndtri(np.linspace(0.0, 1.0, n + 1))  # -inf .. +inf
    dens = np.exp(-0.5 * edges * edges)          # 0 at both infinities
    z = float(sigma_z) * n / np.sqrt(2.0 * np.pi) * (dens[:-1] - dens[1:])
    return np.full(n, float(n_part_tot) / n), z[::-1].copy()
