"""Batched persistent tracking against per-lattice tracking.

The batch kernel runs the tracking kernel's own per-CTA code on tiles of
many lattice variants, so every particle must come out bit-identical to
st_DeviceLattice_track_until on its variant alone (columns compared with
torch.equal): exact and fast arithmetic, direct launches and captured-graph
replays, after autotuning, with empty variants, pre-lost particles and
lattices that mix in beam-beam and space-charge elements.
"""

import numpy as np
import pytest

from sixtracklib_gb300 import lattices

pytestmark = pytest.mark.gpu


def _torch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("GPU tests need a CUDA device")
    return torch


def _variants(mode, n_var=10, seed=5):
    from sixtracklib_gb300.device import DeviceTracker

    torch = _torch()
    rng = np.random.default_rng(seed)
    trk, cols = [], []
    for v in range(n_var):
        e = lattices.variant_ring(seed * 100 + v, int(rng.uniform(200, 3000)))
        n = int(np.exp(rng.uniform(np.log(50), np.log(4000))))
        p = lattices.gaussian_particles(n, seed=v + 1)
        trk.append(DeviceTracker(e, config=f"mode={mode}"))
        cols.append(torch.from_numpy(p.block.copy().view(np.int64)).cuda())
    return trk, cols


def _reference(trk, cols, until):
    out = []
    for t, c in zip(trk, cols):
        r = c.clone()
        assert t.track_until(r, until) == 0
        out.append(r)
    return out


@pytest.mark.parametrize("mode", ["exact", "fast"])
def test_batch_matches_per_lattice(mode):
    torch = _torch()
    from sixtracklib_gb300.batch import BatchTracker

    trk, cols = _variants(mode)
    ref = _reference(trk, cols, 6)
    work = [c.clone() for c in cols]
    bt = BatchTracker(trk, config="threads_per_block=64 stages=3 turns_per_launch=4")
    bt.set_particles(work)
    assert bt.track_until(0, 6) == 0
    torch.cuda.synchronize()
    for w, r in zip(work, ref):
        assert torch.equal(w, r)
    assert sum(int((r[20] == 0).sum()) for r in ref) > 0  # losses are covered


def test_graph_replay_matches_per_lattice():
    torch = _torch()
    from sixtracklib_gb300.batch import BatchTracker

    trk, cols = _variants("fast", seed=9)
    ref = _reference(trk, cols, 6)
    work = [c.clone() for c in cols]
    bt = BatchTracker(trk, config="turns_per_launch=1")
    bt.set_particles(work)
    bt.capture(2)
    bt.set_turn(0)
    for _ in range(3):
        bt.replay()
    assert bt.status() == 0
    for w, r in zip(work, ref):
        assert torch.equal(w, r)


def test_autotune_keeps_particles_and_results():
    torch = _torch()
    from sixtracklib_gb300.batch import BatchTracker

    trk, cols = _variants("fast", seed=13)
    ref = _reference(trk, cols, 4)
    work = [c.clone() for c in cols]
    bt = BatchTracker(trk)
    bt.set_particles(work)
    ms = bt.autotune(sample_fraction=0.25, trial_turns=2)
    assert ms > 0
    for w, c in zip(work, cols):
        assert torch.equal(w, c)  # the autotuner works on a copy
    sh = bt.shape
    assert sh["threads_per_block"] in (64, 128, 256) and 2 <= sh["stages"] <= 8
    assert bt.track_until(0, 4) == 0
    for w, r in zip(work, ref):
        assert torch.equal(w, r)


def test_batch_edge_cases():
    torch = _torch()
    from sixtracklib_gb300.batch import BatchTracker
    from sixtracklib_gb300.device import DeviceTracker

    trk, cols = _variants("exact", n_var=4, seed=21)
    # a lattice with beam-beam and space charge; an empty particle block;
    # pre-lost particles and particles already a few turns ahead
    trk.append(DeviceTracker(lattices.bb_sc_ring(n_sc=20), config="mode=exact"))
    cols.append(torch.from_numpy(lattices.gaussian_particles(300, seed=3).block.copy()
                                 .view(np.int64)).cuda())
    trk.append(DeviceTracker(lattices.fodo_ring(), config="mode=exact"))
    cols.append(torch.zeros((21, 0), dtype=torch.int64, device="cuda"))
    cols[0][20, :7] = 0
    cols[1][19, :5] = 3
    ref = _reference(trk, cols, 5)
    work = [c.clone() for c in cols]
    bt = BatchTracker(trk, config="threads_per_block=128 blocks_per_sm=1 stages=8")
    bt.set_particles(work)
    assert bt.track_until(0, 5) == 0
    for w, r in zip(work, ref):
        assert torch.equal(w, r)


def test_batch_rejects_bad_input():
    torch = _torch()
    from sixtracklib_gb300.batch import BatchTracker
    from sixtracklib_gb300.beam_elements import Elements
    from sixtracklib_gb300.device import DeviceTracker

    e = DeviceTracker(Elements(), config="mode=exact")
    f = DeviceTracker(lattices.fodo_ring(), config="mode=fast")
    g = DeviceTracker(lattices.fodo_ring(), config="mode=exact")
    with pytest.raises(RuntimeError, match="one arithmetic mode"):
        BatchTracker([f, g])
    with pytest.raises(RuntimeError, match="threads_per_block"):
        BatchTracker([g], config="threads_per_block=48")
    bt = BatchTracker([e, g])
    c = torch.from_numpy(lattices.gaussian_particles(10, seed=1).block.copy()
                         .view(np.int64)).cuda()
    with pytest.raises(RuntimeError, match="empty lattice"):
        bt.set_particles([c, c.clone()])
