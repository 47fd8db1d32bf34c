"""The reverse-mode adjoint on the GPU against the dual-number oracle and
central finite differences.

Loss: L = sum over particles and coordinates of w * u_final with random
weights w (scaled by each coordinate's spread), so that dL/du0 and dL/dk
test every entry of the Jacobian; lost particles take part (their gradient
flows back from the element where they were lost).  The dual-number pass
(oracle/dual.py, pinned against the C oracle and finite differences on the
CPU) differs from the adjoint only by rounding: agreement is required to
1e-9 relative to the largest entry of each gradient row.  Central finite
differences of the GPU tracking itself use h = 1e-7 relative for the
quadrupole strengths, whose gradient they resolve to ~1e-8, and h = 1e-3
relative for the weakly coupled sextupole strengths (at 1e-7 their
difference quotient is dominated by the tracking's rounding noise):
agreement within 1e-6 relative.
"""

import os
from math import factorial

import numpy as np
import pytest

from oracle import dual
from sixtracklib_gb300 import lattices
from sixtracklib_gb300.particles import COL

from .adjoint_cases import misc_ring

pytestmark = pytest.mark.gpu

SIGMA = np.array([1e-3, 1e-5, 1e-3, 1e-5, 0.05, 1e-4])
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _torch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("GPU tests need a CUDA device")
    return torch


def _kind(p):
    return -1 if p[1] == "voltage" else 2 * int(p[2]) + (p[1] == "ksl")


def _scale(p):
    return 1.0 if p[1] == "voltage" else 1.0 / factorial(int(p[2]))


def _beam(n, seed, n_lost=8):
    p = lattices.gaussian_particles(n, seed=seed)
    blk = p.block.copy()
    blk.view(np.float64)[COL["x"], :n_lost] = np.linspace(0.013, 0.019, n_lost)
    return blk


def _dual_grads(e, params, blk, T, w):
    kinds = [(int(p[0]), _kind(p)) for p in params]
    vals, ders, st, at, ae = dual.track_until(e, blk.copy(), T, params=kinds)
    g_coords = np.einsum("rn,crn->cn", w, ders[:6])
    g_params = np.einsum("rn,jrn->j", w, ders[6:]) * np.array([_scale(p) for p in params])
    return g_coords, g_params, vals, st


def _gpu_grads(e, params, blk, T, w, config="mode=exact", every=7, reconstruct="inverse"):
    torch = _torch()
    from sixtracklib_gb300.autodiff import DifferentiableLattice, coordinates

    lat = DifferentiableLattice(e, params, config)
    cols = torch.from_numpy(blk.view(np.int64).copy()).cuda()
    coords = coordinates(cols).clone().requires_grad_(True)
    values = torch.tensor(lat.initial_values, dtype=torch.float64, device="cuda",
                          requires_grad=True)
    out, state = lat.track(coords, values, cols, T, checkpoint_every=every,
                           reconstruct=reconstruct)
    loss = (torch.from_numpy(w).cuda() * out).sum()
    loss.backward()
    return (coords.grad.cpu().numpy(), values.grad.cpu().numpy(),
            out.detach().cpu().numpy(), state.cpu().numpy())


def _rel_rows(a, b):
    return np.max(np.abs(a - b), axis=-1) / np.max(np.abs(b), axis=-1)


@pytest.mark.parametrize("reconstruct", ["inverse", "recompute"])
@pytest.mark.parametrize("case", ["fodo", "misc"])
def test_adjoint_matches_dual_numbers(case, reconstruct):
    if case == "fodo":
        e, params = lattices.learnable_fodo_ring()
        T, n = 30, 600
    else:
        e, params = misc_ring()
        T, n = 20, 400
    blk = _beam(n, seed=21)
    w = np.random.default_rng(2).normal(size=(6, n)) / SIGMA[:, None]
    gc_d, gp_d, vals_d, st_d = _dual_grads(e, params, blk, T, w)
    gc, gp, vals, st = _gpu_grads(e, params, blk, T, w, reconstruct=reconstruct)
    assert np.array_equal(st, st_d)
    assert 0 < (st == 0).sum() < n
    np.testing.assert_allclose(vals, vals_d, rtol=1e-12, atol=1e-18)
    assert np.all(_rel_rows(gc, gc_d) < 1e-9), _rel_rows(gc, gc_d)
    assert np.max(np.abs(gp - gp_d) / np.abs(gp_d)) < 1e-8, (gp, gp_d)


@pytest.mark.parametrize("p0c", [7e12, 20e9])
def test_field_kick_adjoints_match_dual_numbers(p0c):
    """RF multipole, 4D beam-beam (round and elliptic), coasting, q-Gaussian
    (q = 1, 1.2, 0.8) and interpolated (linear, cubic, fallback) space charge:
    gradients of the coordinates and of the strengths within 1e-9 of the
    dual-number pass."""
    from .adjoint_cases import field_ring

    e, params, tables = field_ring()
    T, n = 8, 300
    blk = lattices.gaussian_particles(n, seed=31, sz=0.08, p0c=p0c).block.copy()
    w = np.random.default_rng(6).normal(size=(6, n)) / SIGMA[:, None]
    gc_d, gp_d, vals_d, st_d = _dual_grads(e, params, blk, T, w)
    for reconstruct in ("inverse", "recompute"):
        gc, gp, vals, st = _gpu_grads(e, params, blk, T, w, every=3, reconstruct=reconstruct)
        assert np.array_equal(st, st_d)
        np.testing.assert_allclose(vals, vals_d, rtol=1e-11, atol=1e-20)
        assert np.all(_rel_rows(gc, gc_d) < 1e-9), _rel_rows(gc, gc_d)
        assert np.max(np.abs(gp - gp_d) / np.abs(gp_d)) < 1e-8, (gp, gp_d)
    del tables


@pytest.mark.parametrize("p0c", [7e12, 20e9])
def test_beam_beam_6d_adjoint_matches_dual_numbers(p0c):
    """6D beam-beam: round uncoupled, coupled elliptic and head-on elliptic
    strong beams with crossing angles, offsets and dipolar subtraction
    (tests/adjoint_cases.bb6d_ring); gradients of the coordinates and of the
    ring's strengths within 1e-9 of the dual-number pass, with the
    reconstruction by inverse maps and by recomputed turns."""
    from .adjoint_cases import bb6d_ring

    e, params = bb6d_ring(p0c)
    T, n = 8, 300
    blk = lattices.gaussian_particles(n, seed=31, sz=0.08, p0c=p0c).block.copy()
    w = np.random.default_rng(6).normal(size=(6, n)) / SIGMA[:, None]
    gc_d, gp_d, vals_d, st_d = _dual_grads(e, params, blk, T, w)
    for reconstruct in ("inverse", "recompute"):
        gc, gp, vals, st = _gpu_grads(e, params, blk, T, w, every=3, reconstruct=reconstruct)
        assert np.array_equal(st, st_d)
        np.testing.assert_allclose(vals, vals_d, rtol=1e-11, atol=1e-20)
        assert np.all(_rel_rows(gc, gc_d) < 1e-9), _rel_rows(gc, gc_d)
        assert np.max(np.abs(gp - gp_d) / np.abs(gp_d)) < 1e-8, (gp, gp_d)


def test_adjoint_fast_mode_matches_dual_numbers():
    e, params = lattices.learnable_fodo_ring()
    T, n = 20, 300
    blk = _beam(n, seed=5, n_lost=0)
    w = np.random.default_rng(3).normal(size=(6, n)) / SIGMA[:, None]
    gc_d, gp_d, _, _ = _dual_grads(e, params, blk, T, w)
    gc, gp, _, _ = _gpu_grads(e, params, blk, T, w, config="mode=fast")
    assert np.all(_rel_rows(gc, gc_d) < 1e-8)
    assert np.max(np.abs(gp - gp_d) / np.abs(gp_d)) < 1e-7


def test_checkpoint_interval_does_not_change_gradients():
    e, params = lattices.learnable_fodo_ring()
    T, n = 12, 256
    blk = _beam(n, seed=8)
    w = np.random.default_rng(4).normal(size=(6, n)) / SIGMA[:, None]
    # recomputed turn states: the same kernels in the same order
    res = [_gpu_grads(e, params, blk, T, w, every=k, reconstruct="recompute")
           for k in (1, 5, 12, 100)]
    for gc, gp, vals, st in res[1:]:
        assert np.array_equal(gc, res[0][0])
        np.testing.assert_allclose(gp, res[0][1], rtol=1e-12)  # atomics: order varies
        assert np.array_equal(vals, res[0][2])
    # reconstructed states: re-anchored at different turns, rounding-level changes
    for k in (1, 5, 12, 100):
        gc, gp, vals, st = _gpu_grads(e, params, blk, T, w, every=k)
        assert np.array_equal(vals, res[0][2])
        assert np.all(_rel_rows(gc, res[0][0]) < 1e-11)
        assert np.max(np.abs(gp - res[0][1])) < 1e-10 * np.max(np.abs(res[0][1]))


def test_adjoint_vs_central_finite_differences():
    """The workload's own loss shape: mean over surviving particles of
    x^2 + y^2 after the last turn (the lost-particle penalty is piecewise
    constant and has no derivative)."""
    torch = _torch()
    from sixtracklib_gb300.autodiff import DifferentiableLattice, coordinates

    e, params = lattices.learnable_fodo_ring()
    T, n = 50, 4096
    blk = _beam(n, seed=33, n_lost=0)
    lat = DifferentiableLattice(e, params, "mode=exact")
    cols = torch.from_numpy(blk.view(np.int64).copy()).cuda()
    coords = coordinates(cols).clone()
    values = torch.tensor(lat.initial_values, dtype=torch.float64, device="cuda",
                          requires_grad=True)
    out, state = lat.track(coords, values, cols, T, checkpoint_every=10)
    alive = state == 1
    assert bool(alive.all())

    def loss_of(o):
        return ((o[0] ** 2 + o[2] ** 2) * alive).sum() / alive.sum()

    loss_of(out).backward()
    g = values.grad.cpu().numpy()
    v0 = lat.initial_values
    checks = {0: 1e-7, 17: 1e-7, 41: 1e-7, 64: 1e-3, 71: 1e-3}
    with torch.no_grad():
        for j, rel_h in checks.items():
            h = rel_h * abs(v0[j])
            o = []
            for s in (1.0, -1.0):
                v = v0.copy()
                v[j] += s * h
                o.append(lat.track(coords, torch.from_numpy(v).cuda(), cols, T)[0])
            # difference before the reduction: keeps the sum's rounding out
            d = ((o[0][0] - o[1][0]) * (o[0][0] + o[1][0]) +
                 (o[0][2] - o[1][2]) * (o[0][2] + o[1][2])) * alive
            g_fd = float(d.sum() / alive.sum()) / (2 * h)
            assert abs(g[j] - g_fd) <= 1e-6 * abs(g_fd), (j, g[j], g_fd)


def test_lattice_without_adjoint_is_refused():
    """Every map the engine tracks has an adjoint.  A map compiled out of
    the engine (TriCub, as in the reference's default build) fails the
    forward tracking, and the adjoint entry point refuses such a lattice
    before launch."""
    torch = _torch()
    from sixtracklib_gb300.autodiff import DifferentiableLattice, coordinates
    from sixtracklib_gb300.beam_elements import TYPE_TRICUB

    e = lattices.fodo_ring()
    e.TriCub(length=0.1)
    assert e.cbuffer.objects[-1].typeid == TYPE_TRICUB
    lat = DifferentiableLattice(e, [])
    blk = _beam(64, seed=1, n_lost=0)
    cols = torch.from_numpy(blk.view(np.int64).copy()).cuda()
    coords = coordinates(cols).clone().requires_grad_(True)
    with pytest.raises(RuntimeError, match="tracking failed"):
        lat.track(coords, torch.zeros(0, dtype=torch.float64, device="cuda"), cols, 2)
    lam = torch.ones((6, 64), dtype=torch.float64, device="cuda")
    with pytest.raises(RuntimeError, match="without an adjoint"):
        lat.adjoint_turns(cols, cols.clone(), lam, 0, 1)


# ------------------------------------------- the workload at its full length
def _fixture_1000():
    return np.load(os.path.join(GOLDEN, "adjoint_fodo_1000.npz"))


def _track_1000(lat, blk, reconstruct, turns=1000, every=100):
    torch = _torch()
    from sixtracklib_gb300.autodiff import coordinates

    cols = torch.from_numpy(blk.view(np.int64).copy()).cuda()
    coords = coordinates(cols).clone().requires_grad_(True)
    values = torch.tensor(lat.initial_values, dtype=torch.float64, device="cuda",
                          requires_grad=True)
    out, state = lat.track(coords, values, cols, turns, checkpoint_every=every,
                           reconstruct=reconstruct)
    return coords, values, out, state


@pytest.mark.parametrize("reconstruct", ["inverse", "recompute"])
def test_adjoint_1000_turns_matches_dual_numbers(reconstruct):
    """The differentiable-tracking workload at its full length: the learnable
    FODO ring (64 quad strengths, 16 sextupoles), 1,000 turns, a checkpoint
    every 100 turns, 256 particles of which 8 start near the LimitRect edge
    and are lost during the run.  Gradients with respect to the initial
    coordinates and the 80 strengths against the dual-number pass
    (tests/golden/adjoint_fodo_1000.npz, made by make_golden.py --adjoint):
    for a random linear functional of the final coordinates and for the
    workload's objective (autodiff.orbit_loss: mean x^2 + y^2 of the
    survivors plus the smooth aperture penalty), within 1e-9 of the largest
    entry of each gradient row."""
    torch = _torch()
    from sixtracklib_gb300.autodiff import DifferentiableLattice, aperture_shapes, orbit_loss

    d = _fixture_1000()
    e, params = lattices.learnable_fodo_ring()
    lat = DifferentiableLattice(e, params, "mode=exact")
    shapes = aperture_shapes(e)
    assert 0 < int((d["state"] == 0).sum()) < d["state"].size
    for objective in ("linear", "loss"):
        coords, values, out, state = _track_1000(lat, d["initial"], reconstruct)
        st = state.cpu().numpy()
        assert np.array_equal(st, d["state"])
        vals = out.detach().cpu().numpy()
        assert np.all(_rel_rows(vals, d["values"]) < 1e-11), _rel_rows(vals, d["values"])
        if objective == "linear":
            loss = (torch.from_numpy(d["weights"]).cuda() * out).sum()
        else:
            loss = orbit_loss(out, state, shapes)
            assert abs(loss.item() - float(d["loss"])) <= 1e-11 * abs(float(d["loss"]))
        loss.backward()
        gc, gp = coords.grad.cpu().numpy(), values.grad.cpu().numpy()
        gc_d, gp_d = d[objective + "_grad_coords"], d[objective + "_grad_params"]
        rc = _rel_rows(gc, gc_d)
        rp = np.max(np.abs(gp - gp_d)) / np.max(np.abs(gp_d))
        print(f"{reconstruct} {objective}: coordinate rows {rc.max():.2e}, strengths {rp:.2e}")
        assert np.all(rc < 1e-9), rc
        assert rp < 1e-9, rp


def _fd_check(lat, blk, loss_fn, checks, turns=1000, every=100):
    """Central differences of GPU tracking for the parameters `checks`
    ({index: relative step}) against the adjoint's gradient, within 1e-6
    relative.  Every particle must be lost at the same turn and element in
    the +h and -h runs (the difference quotient is then that of a smooth
    function)."""
    torch = _torch()
    from sixtracklib_gb300.autodiff import coordinates

    cols = torch.from_numpy(blk.view(np.int64).copy()).cuda()
    coords = coordinates(cols).clone()
    values = torch.tensor(lat.initial_values, dtype=torch.float64, device="cuda",
                          requires_grad=True)
    out, state = lat.track(coords, values, cols, turns, checkpoint_every=every)
    loss_fn(out, state).backward()
    g = values.grad.cpu().numpy()
    v0 = lat.initial_values
    worst = 0.0
    with torch.no_grad():
        for j, rel_h in checks.items():
            h = rel_h * abs(v0[j])
            runs, where = [], []
            for s in (1.0, -1.0):
                v = v0.copy()
                v[j] += s * h
                o, stt = lat.track(coords, torch.from_numpy(v).cuda(), cols, turns,
                                   checkpoint_every=every)
                runs.append((o, stt))
                c = cols.clone()  # where each particle stopped (state, turn, element)
                lat.set_values(v)
                assert lat.tracker.track_until(c, turns) == 0
                where.append(c[18:21].clone())
            assert torch.equal(runs[0][1], state) and torch.equal(runs[1][1], state)
            assert torch.equal(where[0], where[1]), "a loss moved between the +h and -h runs"
            g_fd = loss_fn(runs[0][0], state, runs[1][0]) / (2 * h)
            rel = abs(g[j] - g_fd) / abs(g_fd)
            worst = max(worst, rel)
            assert rel <= 1e-6, (j, g[j], g_fd)
    return worst


def _orbit_loss_difference(shapes, weight=1e-3):
    """orbit_loss, and the difference of its values at two final states
    taken before the reductions (so that the sums' rounding stays out of the
    difference quotient)."""
    from sixtracklib_gb300.autodiff import aperture_penalty, orbit_loss

    def fn(out, state, other=None):
        if other is None:
            return orbit_loss(out, state, shapes, penalty_weight=weight)
        alive = state == 1
        core = ((out[0] - other[0]) * (out[0] + other[0]) +
                (out[2] - other[2]) * (out[2] + other[2])) * alive
        pen = aperture_penalty(out, shapes) - aperture_penalty(other, shapes)
        return float(core.sum() / alive.sum() + weight * pen.mean())
    return fn


def test_adjoint_1000_turns_vs_finite_differences():
    """The workload's objective (mean x^2 + y^2 of the survivors plus the
    smooth aperture penalty) over 1,000 turns with a checkpoint every 100:
    the adjoint's derivatives with respect to four quad strengths (central
    differences with h = 1e-7 relative) and two sextupole strengths
    (h = 1e-3 relative: their effect on the coordinates is ~1e6 times weaker,
    and at 1e-7 the quotient is the tracking's rounding noise) within 1e-6
    relative."""
    from sixtracklib_gb300.autodiff import DifferentiableLattice, aperture_shapes

    d = _fixture_1000()
    e, params = lattices.learnable_fodo_ring()
    lat = DifferentiableLattice(e, params, "mode=exact")
    worst = _fd_check(lat, d["initial"], _orbit_loss_difference(aperture_shapes(e)),
                      {0: 1e-7, 17: 1e-7, 41: 1e-7, 63: 1e-7, 64: 1e-3, 79: 1e-3})
    print(f"orbit loss, 1000 turns: adjoint vs central differences {worst:.2e}")


def test_aperture_penalty_adjoint_vs_finite_differences():
    """The smooth lost-particle penalty alone (its derivative reaches the lost
    particles through the adjoint from the element where each was lost):
    central differences of the mean penalty over 1,000 turns against the
    adjoint, within 1e-6 relative, for four quad strengths."""
    from sixtracklib_gb300.autodiff import (DifferentiableLattice, aperture_penalty,
                                            aperture_shapes)

    d = _fixture_1000()
    e, params = lattices.learnable_fodo_ring()
    lat = DifferentiableLattice(e, params, "mode=exact")
    shapes = aperture_shapes(e)

    def fn(out, state, other=None):
        if other is None:
            return aperture_penalty(out, shapes).mean()
        return float((aperture_penalty(out, shapes) - aperture_penalty(other, shapes)).mean())

    worst = _fd_check(lat, d["initial"], fn, {3: 1e-7, 22: 1e-7, 40: 1e-7, 61: 1e-7})
    print(f"aperture penalty, 1000 turns: adjoint vs central differences {worst:.2e}")
