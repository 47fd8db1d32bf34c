"""Small self-checking runs of the engine's kernels, for profiling.

    python -m sixtracklib_gb300.run_case adjoint <particles> <turns> <exact|fast>
        one forward + backward of differentiable tracking on the learnable
        FODO ring (loss: mean x^2 + y^2; one checkpoint segment, so one
        adjoint launch);
    python -m sixtracklib_gb300.run_case batch <variants> <turns>
        one batched call over lattice variants of 500-4000 elements with
        1024-32768 particles each, checked bit for bit against per-lattice
        tracking;
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


def bbsc(n: int, turns: int) -> None:
    for r in bbsc_measure(n, turns):
        print(f"bbsc {r['beams']:<33} {r['mode']:<5} {r['particles']} particles: "
              f"{r['ms_per_turn']:.2f} ms/turn, {r['value']:.3e} PET/s")


def main(argv) -> None:
    if len(argv) >= 1 and argv[0] == "adjoint":
        adjoint(int(argv[1]), int(argv[2]), argv[3])
    elif len(argv) >= 1 and argv[0] == "batch":
        batch(int(argv[1]), int(argv[2]))
    elif len(argv) >= 1 and argv[0] == "bbsc":
        bbsc(int(argv[1]), int(argv[2]))
    else:
        raise SystemExit(__doc__)


if __name__ == "__main__":
    main(sys.argv[1:])
