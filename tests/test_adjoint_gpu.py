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

from math import factorial

import numpy as np
import pytest

from oracle import dual
from sixtracklib_gb300 import lattices
from sixtracklib_gb300.particles import COL

from .adjoint_cases import misc_ring

pytestmark = pytest.mark.gpu

SIGMA = np.array([1e-3, 1e-5, 1e-3, 1e-5, 0.05, 1e-4])


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
