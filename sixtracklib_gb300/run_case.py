"""Small self-checking runs of the engine's kernels, for profiling.

    python -m sixtracklib_gb300.run_case adjoint <particles> <turns> <exact|fast>
        one forward + backward of differentiable tracking on the learnable
        FODO ring (loss: mean x^2 + y^2; one checkpoint segment, so one
        adjoint launch);
    python -m sixtracklib_gb300.run_case batch <variants> <turns>
        one batched call over lattice variants of 500-4000 elements with
        1024-32768 particles each, checked bit for bit against per-lattice
        tracking.

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


def main(argv) -> None:
    if len(argv) >= 1 and argv[0] == "adjoint":
        adjoint(int(argv[1]), int(argv[2]), argv[3])
    elif len(argv) >= 1 and argv[0] == "batch":
        batch(int(argv[1]), int(argv[2]))
    else:
        raise SystemExit(__doc__)


if __name__ == "__main__":
    main(sys.argv[1:])
