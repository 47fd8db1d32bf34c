"""Small self-checking runs of the engine's kernels, for profiling.

    python -m sixtracklib_gb300.run_case adjoint <particles> <turns> <exact|fast>
        one forward + backward of differentiable tracking on the learnable
        FODO ring (loss: mean x^2 + y^2; one checkpoint segment, so one
        adjoint launch);
    python -m sixtracklib_gb300.run_case batch <variants> <turns>
        one batched call over lattice variants of 500-4000 elements with
        1024-32768 particles each, checked bit for bit against per-lattice
        tracking;
    python -m sixtracklib_gb300.run_case elements <particles>
        one turn (fast arithmetic) of each of: the FODO ring, and the FODO
        ring plus 200 round / 200 elliptic q-Gaussian space-charge kicks,
        50 round 4D beam-beam kicks, 4 round / 4 elliptic 6D beam-beam
        elements of 21 slices -- under a profiler's instruction counters,
        the differences to the plain ring give each element's cost;
    python -m sixtracklib_gb300.run_case bbsc <particles> <turns>
        the beam-beam and space-charge mix (FODO ring + 4 BeamBeam6D of 21
        slices + 4 BeamBeam4D + 200 q-Gaussian space-charge kicks), round
        and elliptic strong beams, Gaussian protons: <turns> timed turns
        after 2 warm-up turns, fast and exact arithmetic.

Each prints one line and exits non-zero if its check fails.
"""

from __future__ import annotations

import sys

import numpy as np


def adjoint(n: int, turns: int, mode: str) -> None:
    import torch

    from . import lattices
    from .autodiff import DifferentiableLattice, coordinates

    ring, params = lattices.learnable_fodo_ring()
    lat = DifferentiableLattice(ring, params, f"mode={mode}")
    cols = torch.from_numpy(lattices.gaussian_particles(n, seed=1).block.copy()
                            .view(np.int64)).cuda()
    coords = coordinates(cols).clone().requires_grad_(True)
    values = torch.tensor(lat.initial_values, dtype=torch.float64, device="cuda",
                          requires_grad=True)
    out, _ = lat.track(coords, values, cols, turns, checkpoint_every=turns)
    (out[0] ** 2 + out[2] ** 2).mean().backward()
    torch.cuda.synchronize()
    g = values.grad
    if not bool(torch.isfinite(g).all()) or float(g.abs().max()) == 0.0:
        raise SystemExit("adjoint: gradient not finite or zero")
    print(f"adjoint {n} particles x {turns} turns ({mode}): |grad| = {float(g.norm()):.6e}")


def batch(n_variants: int, turns: int) -> None:
    import torch

    from . import lattices
    from .batch import BatchTracker
    from .device import DeviceTracker

    specs = lattices.batch_specs(n_variants=n_variants, particles=(1024, 32768),
                                 elements=(500, 4000))
    trk = [DeviceTracker(lattices.variant_ring(s, e), config="mode=fast")
           for s, e, _, _ in specs]
    cols = [torch.from_numpy(lattices.gaussian_particles(n, seed=ps).block.copy()
                             .view(np.int64)).cuda() for _, _, n, ps in specs]
    ref = [c.clone() for c in cols]
    for t, r in zip(trk, ref):
        if t.track_until(r, turns) != 0:
            raise SystemExit("per-lattice tracking failed")
    bt = BatchTracker(trk, config="threads_per_block=64 blocks_per_sm=2 stages=3")
    bt.set_particles(cols)
    if bt.track_until(0, turns) != 0:
        raise SystemExit("batched tracking failed")
    if not all(torch.equal(c, r) for c, r in zip(cols, ref)):
        raise SystemExit("batched != per-lattice")
    print(f"batch {n_variants} variants, {sum(c.shape[1] for c in cols)} particles x "
          f"{turns} turns: bit-identical to per-lattice tracking")


def bbsc_measure(n: int, turns: int, modes=("fast", "exact")) -> list:
    """Particle-element-turns/s of the beam-beam and space-charge mix
    (lattices.bb_sc_ring) with round and with elliptic strong beams."""
    import torch

    from . import lattices
    from .device import DeviceTracker

    out = []
    stream = torch.cuda.current_stream()
    for elliptic in (False, True):
        ring = lattices.bb_sc_ring(elliptic=elliptic)
        block = lattices.gaussian_particles(n, seed=3).block
        for mode in modes:
            trk = DeviceTracker(ring, config=f"mode={mode}")
            cols = torch.from_numpy(block.copy().view(np.int64)).cuda()
            if trk.track_until(cols, 2) != 0:
                raise SystemExit("bbsc: tracking failed")
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            a.record(stream)
            trk.launch_until(cols, 2 + turns)
            b.record(stream)
            torch.cuda.synchronize()
            if trk.last_status() != 0:
                raise SystemExit("bbsc: tracking failed")
            sec = a.elapsed_time(b) / 1e3
            alive = int((cols[20] == 1).sum())
            out.append({"beams": "elliptic (sigma_y = 1.3 sigma_x)" if elliptic else "round",
                        "mode": mode, "particles": n, "alive": alive,
                        "elements": len(ring), "turns_timed": turns,
                        "ms_per_turn": sec / turns * 1e3,
                        "value": alive * len(ring) * turns / sec})
    return out


def element_cost_lattices() -> dict:
    """The FODO ring with one kind of beam-field element added (see the
    module doc); strong beams of 16.7 um (beam-beam) and 1 mm (space
    charge), as in lattices.bb_sc_ring."""
    from math import erf, sqrt

    from . import lattices
    from .beam_elements import QELEM, bb6d_data

    def sc(ell):
        e = lattices.fodo_ring()
        for _ in range(200):
            e.SCQGaussProfile(number_of_particles=1e11, bunchlength_rms=0.1, sigma_x=1e-3,
                              sigma_y=1.2e-3 if ell else 1e-3, length=1.0, x_co=0.0, y_co=0.0,
                              min_sigma_diff=1e-10, q_param=1.0, enabled=1)
        return e

    def bb4d():
        e = lattices.fodo_ring()
        for _ in range(50):
            e.BeamBeam4D(charge=1.15e11, sigma_x=16.7e-6, sigma_y=16.7e-6, beta_r=1.0,
                         min_sigma_diff=1e-10, x_bb=1e-6, y_bb=-1e-6, d_px=0.0, d_py=0.0,
                         enabled=1.0)
        return e

    def bb6d(ell, ns=21, sz=0.0755):
        edges = np.linspace(0.0, 1.0, ns + 1)
        z = np.zeros(ns)
        for i in range(ns):  # equal-charge slices of a Gaussian bunch
            lo, hi, mid = -8.0, 8.0, 0.5 * (edges[i] + edges[i + 1])
            for _ in range(80):
                m = 0.5 * (lo + hi)
                lo, hi = (m, hi) if 0.5 * (1 + erf(m / sqrt(2))) < mid else (lo, m)
            z[i] = 0.5 * (lo + hi) * sz
        sx = 16.7e-6
        sy = sx * (1.3 if ell else 1.0)
        e = lattices.fodo_ring()
        for _ in range(4):
            e.BeamBeam6D(data=bb6d_data(
                q_part=QELEM, phi=1.5e-4, alpha=0.3, delta_x=1e-6, delta_y=-1e-6,
                n_part_per_slice=np.full(ns, 1.15e11 / ns), z_slices=z,
                sigmas=(sx * sx, 0, 0, 0, 1e-12, 0, 0, sy * sy, 0, 1e-12)))
        return e

    return {"fodo": lattices.fodo_ring(), "sc_round": sc(False), "bb4d_round": bb4d(),
            "bb6d_round": bb6d(False), "sc_elliptic": sc(True), "bb6d_elliptic": bb6d(True)}


def elements(n: int) -> None:
    import torch

    from . import lattices
    from .device import DeviceTracker

    block = lattices.gaussian_particles(n, seed=3).block
    for name, ring in element_cost_lattices().items():
        trk = DeviceTracker(ring, config="mode=fast")
        cols = torch.from_numpy(block.copy().view(np.int64)).cuda()
        if trk.track_until(cols, 1) != 0:
            raise SystemExit(f"elements: tracking {name} failed")
        torch.cuda.synchronize()
        print(f"elements {name:<14} {len(ring)} elements, {int((cols[20] == 1).sum())} alive")


def bbsc(n: int, turns: int) -> None:
    for r in bbsc_measure(n, turns):
        print(f"bbsc {r['beams']:<33} {r['mode']:<5} {r['particles']} particles: "
              f"{r['ms_per_turn']:.2f} ms/turn, {r['value']:.3e} PET/s")


def main(argv) -> None:
    if len(argv) >= 1 and argv[0] == "adjoint":
        adjoint(int(argv[1]), int(argv[2]), argv[3])
    elif len(argv) >= 1 and argv[0] == "batch":
        batch(int(argv[1]), int(argv[2]))
    elif len(argv) >= 1 and argv[0] == "elements":
        elements(int(argv[1]))
    elif len(argv) >= 1 and argv[0] == "bbsc":
        bbsc(int(argv[1]), int(argv[2]))
    else:
        raise SystemExit(__doc__)


if __name__ == "__main__":
    main(sys.argv[1:])
