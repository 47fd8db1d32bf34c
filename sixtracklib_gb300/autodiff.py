"""Differentiable until-turn tracking (reverse mode) for PyTorch.

The reference tracks but does not differentiate.  This module adds
gradients of a loss on the final coordinates with respect to

* the initial coordinates (x, px, y, py, zeta, delta) of every particle, and
* chosen element parameters: multipole ``knl[k]`` / ``ksl[k]`` and cavity
  ``voltage``,

through :class:`TrackFunction`, a ``torch.autograd.Function`` whose forward
is the engine's until-turn tracking kernel and whose backward is the
engine's hand-written adjoint kernel (``st_DeviceLattice_adjoint_turns``),
last checkpoint segment first.

Memory: the forward stores the particle columns every ``checkpoint_every``
turns (``turns / checkpoint_every + 1`` column blocks of ``168 * n`` bytes).
The backward works one segment at a time, either reversing it in one launch
from the states at its two ends (``reconstruct="inverse"``: the maps are
inverted element by element) or recomputing its turn-boundary states from
the checkpoint first (``reconstruct="recompute"``: ``checkpoint_every + 1``
more blocks; the tracking kernel is deterministic, so the recomputed states
are the forward's states bit for bit).

Conventions: delta is the independent longitudinal coordinate; rpp, rvv and
psigma follow it as NS(Particles_update_delta_value) defines them
(particles.h:5459-5496).  Lost particles keep the coordinates they had when
they were lost (the reference's convention); their gradient flows back from
there.  Apertures contribute no derivative to the tracking itself; a loss
that should see particle losses adds :func:`aperture_penalty`, a smooth
function of the final (or loss-point) coordinates.
"""

from __future__ import annotations

import ctypes as C
from math import factorial

import numpy as np

from . import _native
from .beam_elements import Cavity, Elements, Multipole
from .device import DeviceTracker, _check_cols, _stream_handle
from .particles import COL

COORDS = ("x", "px", "y", "py", "zeta", "delta")
COORD_ROWS = tuple(COL[c] for c in COORDS)


def parameter_table(elements: Elements, params) -> dict:
    """Resolve learnable parameters against a lattice.

    ``params``: ``(element_index, "knl" | "ksl", k)`` or ``(element_index,
    "voltage")``.  Returns per parameter its element, its kind (the ``bal``
    index 2k or 2k+1, or -1 for a cavity voltage), the factor from the
    user's value to the stored one (1/k! for ``knl`` / ``ksl``) and the
    current value; and the per-element table the adjoint kernel reads:
    ``begin`` (num_elements + 1 offsets), ``entry_kind`` and ``entry_id``
    (the parameter each entry belongs to), entries sorted by element."""
    objs = elements.get_elements()
    kinds, elems, scales, init = [], [], [], []
    for p in params:
        e = int(p[0])
        if not 0 <= e < len(objs):
            raise IndexError(f"element index {e} out of range")
        obj = objs[e]
        name = p[1]
        if name in ("knl", "ksl"):
            if not isinstance(obj, Multipole):
                raise TypeError(f"element {e} is not a Multipole")
            k = int(p[2])
            if not 0 <= k <= int(obj.order):
                raise ValueError(f"element {e}: order {obj.order} has no {name}[{k}]")
            kind = 2 * k + (name == "ksl")
            scale = 1.0 / factorial(k)  # bal[2k] = knl[k] / k!
            value = float(obj.bal[kind]) / scale
        elif name == "voltage":
            if not isinstance(obj, Cavity):
                raise TypeError(f"element {e} is not a Cavity")
            kind, scale, value = -1, 1.0, float(obj.voltage)
        else:
            raise ValueError(f"unknown parameter {name!r}")
        elems.append(e)
        kinds.append(kind)
        scales.append(scale)
        init.append(value)
    el = np.asarray(elems, dtype=np.int64)
    ki = np.asarray(kinds, dtype=np.int32)
    n_el = len(objs)
    order = np.argsort(el, kind="stable")
    counts = np.bincount(el, minlength=n_el) if len(elems) else np.zeros(n_el, np.int64)
    begin = np.zeros(n_el + 1, dtype=np.int32)
    begin[1:] = np.cumsum(counts)
    return {"element": el, "kind": ki, "scale": np.asarray(scales, dtype=np.float64),
            "value": np.asarray(init, dtype=np.float64), "begin": begin,
            "entry_kind": ki[order].astype(np.int32), "entry_id": order.astype(np.int32)}


class DifferentiableLattice:
    """A compiled lattice plus the list of its learnable parameters.

    ``params`` is a sequence of ``(element_index, "knl", k)``,
    ``(element_index, "ksl", k)`` or ``(element_index, "voltage")``.
    """

    def __init__(self, elements: Elements, params, config: str | None = "mode=exact"):
        self.params = list(params)
        t = parameter_table(elements, self.params)
        self._elems, self._kinds, self.scales, self.initial_values = (
            t["element"], t["kind"], t["scale"], t["value"])
        self._pbeg, self._pkind, self._pid = t["begin"], t["entry_kind"], t["entry_id"]
        self.tracker = DeviceTracker(elements, config)
        self._lib = _native.load()
        self._dev_tables = {}

    @property
    def num_params(self) -> int:
        return len(self._kinds)

    def _tables(self, device):
        import torch

        key = str(device)
        if key not in self._dev_tables:
            mk = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(device)  # noqa: E731
            self._dev_tables[key] = (mk(self._pbeg), mk(self._pkind), mk(self._pid))
        return self._dev_tables[key]

    def set_values(self, values) -> None:
        """Write parameter values (knl / ksl / voltage units) into the
        compiled lattice."""
        v = np.asarray(values.detach().cpu().numpy() if hasattr(values, "detach") else values,
                       dtype=np.float64).reshape(-1)
        if v.shape[0] != self.num_params:
            raise ValueError(f"expected {self.num_params} parameter values, got {v.shape[0]}")
        if self.num_params == 0:
            return
        bal = np.ascontiguousarray(v * self.scales)
        rc = self._lib.st_DeviceLattice_set_parameters(
            self.tracker._ptr, self.num_params, self._elems.ctypes.data, self._kinds.ctypes.data,
            bal.ctypes.data)
        if rc != 0:
            raise RuntimeError("set_parameters: " + _native.last_error())

    def adjoint_turns(self, start, end, lam, turn_begin: int, turn_end: int, grad=None) -> None:
        """dL/d(coordinates at turn_begin) from dL/d(coordinates at
        turn_end), in place in `lam` (6 x n); parameter contributions added
        to `grad` (dL/d bal or voltage, per parameter), if given.  `start`
        and `end` are the column blocks at the two turns."""
        n = _check_cols(start)
        if _check_cols(end) != n or tuple(lam.shape) != (6, n) or not lam.is_contiguous():
            raise ValueError("adjoint_turns: inconsistent shapes")
        if grad is not None and self.num_params:
            pbeg, pkind, pid = self._tables(start.device)
            tabs = (pbeg.data_ptr(), pkind.data_ptr(), pid.data_ptr(), self.num_params,
                    grad.data_ptr())
        else:
            tabs = (None, None, None, 0, None)
        rc = self._lib.st_DeviceLattice_adjoint_turns(
            self.tracker._ptr, start.data_ptr(), end.data_ptr(), n, int(turn_begin),
            int(turn_end), lam.data_ptr(), *tabs, _stream_handle(start))
        if rc != 0:
            raise RuntimeError("adjoint: " + _native.last_error())

    def track(self, coords, values, cols, until_turn: int, checkpoint_every: int = 100,
              reconstruct: str = "inverse"):
        """Differentiable tracking: ``(final coordinates 6 x n, final state n)``.

        ``reconstruct`` selects how the backward pass obtains the states
        inside a checkpoint segment: ``"inverse"`` reverses the whole segment
        in one launch, reconstructing each element's input by inverting the
        map (no recomputation; the reconstruction is re-anchored at every
        checkpoint); ``"recompute"`` re-tracks the segment from its
        checkpoint storing every turn boundary, then reverses one turn per
        launch (re-anchored every turn, ~1 forward pass more work)."""
        if reconstruct not in ("inverse", "recompute"):
            raise ValueError("reconstruct must be 'inverse' or 'recompute'")
        return TrackFunction.apply(coords, values, self, cols, int(until_turn),
                                   int(checkpoint_every), reconstruct)


def apply_values(elements: Elements, params, values) -> Elements:
    """A copy of `elements` with the listed parameters set to `values`
    (knl / ksl / voltage units): the lattice a training loop exports."""
    values = np.asarray(values, dtype=np.float64).reshape(-1)
    if len(values) != len(params):
        raise ValueError("one value per parameter expected")
    objs = elements.get_elements()
    for p, v in zip(params, values):
        obj = objs[int(p[0])]
        if p[1] == "voltage":
            obj.voltage = float(v)
        else:
            k = int(p[2])
            obj.bal = np.array(obj.bal, dtype=np.float64)
            obj.bal[2 * k + (p[1] == "ksl")] = float(v) / factorial(k)
    out = Elements()
    for obj in objs:
        out.cbuffer.add_object(*obj._encode())
    return out


def aperture_shapes(elements: Elements, x_limit: float = 1.0, y_limit: float = 1.0):
    """The distinct apertures a particle of `elements` can be lost at, as
    ``(kind, parameters)``: ``("rect", (cx, cy, hx, hy))`` for LimitRect
    (be_limit/track.h:90-111) and for the global aperture after drifts
    (be_limit/track.h:54-88, limits x_limit / y_limit), ``("ellipse",
    (a_squ, b_squ))`` for LimitEllipse (be_limit/track.h:113-137); a
    LimitRectEllipse (be_limit/track.h:139-162) contributes both shapes."""
    shapes = {("rect", (0.0, 0.0, float(x_limit), float(y_limit)))}
    for obj in elements.get_elements():
        name = type(obj).__name__
        if name == "LimitRect":
            shapes.add(("rect", (0.5 * (obj.max_x + obj.min_x), 0.5 * (obj.max_y + obj.min_y),
                                 0.5 * (obj.max_x - obj.min_x), 0.5 * (obj.max_y - obj.min_y))))
        elif name == "LimitEllipse":
            shapes.add(("ellipse", (float(obj.a_squ), float(obj.b_squ))))
        elif name == "LimitRectEllipse":
            shapes.add(("rect", (0.0, 0.0, float(obj.max_x), float(obj.max_y))))
            shapes.add(("ellipse", (float(obj.a_squ), float(obj.b_squ))))
    return sorted(shapes)


def aperture_penalty(coords, shapes, width: float = 0.05, power: int = 16):
    """Smooth lost-particle penalty, one value per particle.

    The reference's loss is a step: a particle is lost where its state
    becomes 0 at an aperture (be_limit/track.h:54-162; the loop freezes it
    there, track/track.h:663-666), which has no derivative.  This penalty
    replaces the step by a softplus of each particle's normalised aperture
    coordinate rho (1 on the aperture boundary, 0 on the axis):

        P = width * softplus((rho - 1) / width)

    ~0 deep inside, width * log(2) on the boundary, rho - 1 beyond it.
    rho combines the apertures with a p-norm (power 16), a smooth maximum:
    rho_rect = (|(x - cx) / hx|^p + |(y - cy) / hy|^p)^(1/p) (the rectangle's
    smooth stand-in), rho_ellipse = sqrt(x^2 / a^2 + y^2 / b^2),
    rho = (sum of rho_k^p)^(1/p).  A lost particle keeps the coordinates
    it had at its aperture (rho ~ 1), so the penalty's gradient reaches it
    through the adjoint from the element where it was lost; a surviving
    particle near an edge is pushed inwards.  Non-finite coordinates (a
    particle lost at the global aperture with a NaN / inf coordinate) give
    a constant penalty of `width * log(2)` and no gradient.  The
    derivative is PyTorch's autograd of these expressions.

    `coords` is 6 x n (x, px, y, py, zeta, delta); `shapes` from
    :func:`aperture_shapes`."""
    import torch

    x, y = coords[0], coords[2]
    ok = torch.isfinite(x) & torch.isfinite(y)
    x = torch.where(ok, x, torch.zeros_like(x))
    y = torch.where(ok, y, torch.zeros_like(y))
    acc = torch.zeros_like(x)
    for kind, prm in shapes:
        if kind == "rect":
            cx, cy, hx, hy = prm
            r = (((x - cx) / hx) ** power + ((y - cy) / hy) ** power) ** (1.0 / power)
        else:
            a_squ, b_squ = prm
            r = torch.sqrt(x * x / a_squ + y * y / b_squ)
        acc = acc + r ** power
    rho = acc ** (1.0 / power)
    pen = width * torch.nn.functional.softplus((rho - 1.0) / width)
    return torch.where(ok, pen, torch.full_like(pen, width * float(np.log(2.0))))


def orbit_loss(out, state, shapes, penalty_weight: float = 1e-3, width: float = 0.05):
    """The differentiable-tracking objective: mean over surviving particles
    of x^2 + y^2 after the last turn, plus `penalty_weight` times the mean
    over all particles of :func:`aperture_penalty`."""
    alive = state == 1
    core = ((out[0] ** 2 + out[2] ** 2) * alive).sum() / alive.sum().clamp(min=1)
    return core + penalty_weight * aperture_penalty(out, shapes, width).mean()


def coordinates(cols):
    """The 6 x n coordinate rows (x, px, y, py, zeta, delta) of a column block."""
    return cols.view(dtype=__import__("torch").float64)[list(COORD_ROWS)]


def set_coordinates(cols, coords) -> None:
    """Write x, px, y, py, zeta, delta into a column block and derive rpp,
    rvv, psigma from delta (particles.h:5459-5496)."""
    import torch

    f = cols.view(dtype=torch.float64)
    c = coords.detach().to(torch.float64)
    for r, row in enumerate(COORD_ROWS):
        f[row] = c[r]
    beta0 = f[COL["beta0"]]
    d = c[5]
    db0 = d * beta0
    ptau_beta0 = torch.sqrt(db0 * db0 + 2.0 * db0 * beta0 + 1.0) - 1.0
    opd = 1.0 + d
    f[COL["rvv"]] = opd / (1.0 + ptau_beta0)
    f[COL["rpp"]] = 1.0 / opd
    f[COL["psigma"]] = ptau_beta0 / (beta0 * beta0)


def _start_turn(cols) -> int:
    import torch

    alive = cols[COL["state"]] == 1
    if not bool(alive.any()):
        return int(cols[COL["at_turn"]].max())
    return int(torch.where(alive, cols[COL["at_turn"]], cols[COL["at_turn"]].max()).min())


def _track_checked(lat: DifferentiableLattice, cols, until: int) -> None:
    st = lat.tracker.track_until(cols, until)
    if st != 0:
        raise RuntimeError(f"tracking failed (status {st}): " + _native.last_error())


class TrackFunction:
    """``torch.autograd.Function``: (coords 6 x n, parameter values) ->
    (final coords 6 x n, final state)."""

    _fn = None

    @classmethod
    def apply(cls, *args):
        if cls._fn is None:
            cls._fn = _make_function()
        return cls._fn.apply(*args)


def _make_function():
    import torch

    class _Track(torch.autograd.Function):
        @staticmethod
        def forward(ctx, coords, values, lat, cols, until_turn, every, reconstruct):
            if every < 1:
                raise ValueError("checkpoint_every must be >= 1")
            lat.set_values(values)
            work = cols.clone()
            set_coordinates(work, coords)
            t0 = _start_turn(work)
            ckpts = {t0: work.clone()}
            t = t0
            while t < until_turn:
                t1 = min(t + every, until_turn)
                _track_checked(lat, work, t1)
                t = t1
                if t < until_turn:
                    ckpts[t] = work.clone()
            ckpts[max(t, t0)] = work
            ctx.lat, ctx.ckpts, ctx.every, ctx.reconstruct = lat, ckpts, every, reconstruct
            ctx.values = values.detach().clone() if torch.is_tensor(values) else values
            ctx.coords_dtype = coords.dtype
            out = coordinates(work).clone().to(coords.dtype)
            state = work[COL["state"]].clone()
            ctx.mark_non_differentiable(state)
            return out, state

        @staticmethod
        def backward(ctx, g_out, g_state):
            lat = ctx.lat
            turns = sorted(ctx.ckpts)
            first = ctx.ckpts[turns[0]]
            n, dev = first.shape[1], first.device
            if g_out is None:
                lam = torch.zeros((6, n), dtype=torch.float64, device=dev)
            else:
                lam = g_out.detach().to(torch.float64).contiguous().clone()
            grad = torch.zeros(lat.num_params, dtype=torch.float64, device=dev)
            lat.set_values(ctx.values)
            blocks = None
            for ts, te in reversed(list(zip(turns[:-1], turns[1:]))):
                if ctx.reconstruct == "inverse":
                    lat.adjoint_turns(ctx.ckpts[ts], ctx.ckpts[te], lam, ts, te, grad)
                    continue
                # turn-boundary states of the segment, launched back to back
                if blocks is None or blocks.shape[0] < te - ts + 1:
                    blocks = torch.empty((te - ts + 1,) + tuple(first.shape), dtype=first.dtype,
                                         device=dev)
                blocks[0].copy_(ctx.ckpts[ts])
                for t in range(ts, te):
                    blocks[t - ts + 1].copy_(blocks[t - ts])
                    lat.tracker.launch_until(blocks[t - ts + 1], t + 1)
                st = lat.tracker.last_status()
                if st != 0:
                    raise RuntimeError(f"tracking failed (status {st}): " + _native.last_error())
                for t in range(te - 1, ts - 1, -1):
                    lat.adjoint_turns(blocks[t - ts], blocks[t - ts + 1], lam, t, t + 1, grad)
            g_values = grad * torch.from_numpy(lat.scales).to(dev)
            if torch.is_tensor(ctx.values):
                g_values = g_values.to(ctx.values.dtype)
            return lam.to(ctx.coords_dtype), g_values, None, None, None, None, None

    return _Track
