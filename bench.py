"""Benchmark: FP64 element-by-element tracking throughput on the GPU.

Workload (one "step" = one turn of every particle through the ring):
  the synthetic 20,000-element ring (9,000 drifts, 8,000 multipoles of order
  1-10, 1,000 XYShift, 1,000 SRotation, 16 cavities, 984 elliptic apertures;
  sixtracklib_gb300/lattices.py) tracked with 1,000,000 protons on the polar
  amplitude grid (0-20 sigma x 11 angles, delta ~ U(-3e-4, 3e-4)), FP64.
Metric: particle-element-turns per second (PET/s); every element a live
particle passes counts once (lost particles stop counting where they are lost).

  value       device-resident: columns in HBM, one kernel launch per step;
  e2e         through the C ABI (st_TrackJob_*) with host buffers: each step
              pushes the particle set host->device, tracks, collects back;
  roofline    FP64 pipe: algorithmic FLOPs of the maps (roofline.py) per
              launch / launch time, against the DFMA peak measured in-process;
  cpu_baseline  the CPU oracle (C restatement of the reference loop, OpenMP
              over particles) on a bounded sample of the same workload.
  batched     256 lattice variants (rings built like the synthetic ring, element
              count ~ U(500, 20000), particle count ~ log-uniform(1024, 262144),
              Gaussian 6D): one captured CUDA graph of the persistent batch
              kernel (autotuned launch shape; turns per launch up to 8
              compete) against one plain tracking launch per variant, both
              over the same 20 turns (--batched-turns) after one warm-up turn;
              results compared bit for bit.
  adjoint     the differentiable-tracking workload: the FODO ring with 64
              quadrupole and 16 sextupole strengths as parameters, 65,536
              Gaussian protons, 1,000 turns, a checkpoint every 100 turns;
              loss = mean over surviving particles of x^2 + y^2 plus a
              smooth lost-particle penalty (autodiff.orbit_loss: softplus of
              each particle's normalised aperture coordinate); forward and
              backward timed with CUDA events; ratio = backward / plain
              tracking of the same turns.
  beam_beam_space_charge
              the beam-beam and space-charge mix: the FODO ring plus 4
              BeamBeam6D (21 slices), 4 BeamBeam4D and 200 q-Gaussian
              space-charge kicks, 262,144 Gaussian protons, round and
              elliptic (sigma_y = 1.3 sigma_x) strong beams; 5 turns timed
              with CUDA events after 2 warm-up turns, next to the oracle on
              the host cores on a strided sample of the same particles.
  tricub      the TriCub map enabled (track_tricub=enabled): the FODO ring
              plus 64 TriCub kicks sharing one 100 x 100 x 50 field map,
              262,144 Gaussian protons, 5 turns timed with CUDA events after
              2 warm-up turns (the first call also computes the map's cell
              coefficients on the GPU, timed apart), FP64 roofline with the
              Horner operation count, the oracle on the host cores beside it.

python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
"""

from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-element-turns/s"
WORKLOAD = "synthetic 20k-element ring, 1M particles polar grid, FP64, 1 turn per step"
# DRAM bytes (read + write) of one tracking launch of the default workload
# (1M particles, fast, 128 threads, 2 CTAs/SM), measured with ncu
# (dram__bytes_read.sum + dram__bytes_write.sum, 1 pass; two launches after
# the warm-up: 113.0 and 111.6 MB; profiles/track_kernel_synthetic_ring_20k.md)
TRACK_TRAFFIC_BYTES = 1.123e8


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=6)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--particles", type=int, default=1_000_000)
    ap.add_argument("--mode", default="fast", choices=["fast", "exact"])
    ap.add_argument("--threads", type=int, default=128)
    ap.add_argument("--blocks-per-sm", type=int, default=2)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-bbsc", action="store_true")
    ap.add_argument("--no-tricub", action="store_true")
    ap.add_argument("--tricub-particles", type=int, default=262144)
    ap.add_argument("--tricub-turns", type=int, default=5)
    ap.add_argument("--batch-variants", type=int, default=256)
    ap.add_argument("--batched-turns", type=int, default=20)
    ap.add_argument("--batched-detail", action="store_true",
                    help="also time one plain launch per variant on its own")
    ap.add_argument("--batched-no-tune", action="store_true",
                    help="keep the batch's default launch shape (no autotuning)")
    ap.add_argument("--bbsc-particles", type=int, default=262144)
    ap.add_argument("--bbsc-turns", type=int, default=5)
    ap.add_argument("--adjoint-particles", type=int, default=65536)
    ap.add_argument("--adjoint-turns", type=int, default=1000)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


# ------------------------------------------------------------------ clocks
class ClockSampler:
    """nvidia-smi samples during the timed region (median SM clock, reasons)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=2)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() in ("active", "1", "0x1"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)),
                "reasons": sorted(reasons), "samples": len(sm)}


# -------------------------------------------------------------- workload
def make_workload(n):
    from sixtracklib_gb300 import lattices

    ring = lattices.synthetic_ring()
    parts = lattices.polar_grid_particles(n)
    return ring, parts


def pet_between(before, after, n_elem):
    """Exact particle-element-turns done between two column-block states."""
    import torch

    st0 = before[20]
    t0, t1 = before[19], after[19]
    e0, e1 = before[18], after[18]
    st1 = after[20]
    alive0 = st0 == 1
    turns = (t1 - t0).clamp(min=0)
    lost = alive0 & (st1 == 0)
    pet = torch.where(alive0, turns * n_elem, torch.zeros_like(turns))
    pet = pet + torch.where(lost, (e1 - e0) + 1, torch.zeros_like(turns))
    return int(pet.sum().item())


def host_cpu_model() -> str:
    """The host CPU's model name (/proc/cpuinfo: `model name`, or on Arm the
    implementer / part numbers when no name is given), with the core count."""
    name, impl, part = "", "", ""
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                key, _, val = line.partition(":")
                key, val = key.strip().lower(), val.strip()
                if key == "model name" and not name:
                    name = val
                elif key == "cpu implementer" and not impl:
                    impl = val
                elif key == "cpu part" and not part:
                    part = val
    except OSError:
        pass
    if not name and impl:
        # 0x41 = Arm Ltd; part 0xd4f = Neoverse V2 (the Grace CPU core)
        known = {("0x41", "0xd4f"): "Arm Neoverse V2 (NVIDIA Grace)"}
        name = known.get((impl, part), f"Arm implementer {impl} part {part}")
    import platform

    return f"{name or platform.processor() or platform.machine()}, {os.cpu_count()} cores"


def cpu_baseline(ring, parts, seconds, threads=None, flags=None):
    """Time the oracle (OpenMP over particles) on a sample of the workload
    (map feature flags `flags` as Oracle.set_track_flags takes them)."""
    from oracle.pyoracle import Oracle

    orc = Oracle()
    orc.set_track_flags(*(flags or ()))
    lat = ring.cbuffer.to_image()
    n_elem = len(ring)
    stride = max(1, parts.num_particles // 16384)
    sample = parts.block[:, ::stride][:, :16384].copy()
    n = sample.shape[1]
    t = time.perf_counter()
    b = sample.copy()
    orc.track_until(lat, b, 1)
    dt1 = time.perf_counter() - t
    turns = max(1, int(seconds / max(dt1, 1e-3)))
    b = sample.copy()
    t = time.perf_counter()
    orc.track_until(lat, b, turns)
    dt = time.perf_counter() - t
    alive0 = sample[20].view(np.int64) == 1
    t1 = b[19].view(np.int64)
    st1 = b[20].view(np.int64)
    e1 = b[18].view(np.int64)
    pet = int((alive0 * t1 * n_elem).sum() + ((alive0 & (st1 == 0)) * (e1 + 1)).sum())
    cores = orc.set_num_threads(0)
    out = {"value": pet / dt, "unit": METRIC, "cores": cores, "kind": "port",
           "cpu": host_cpu_model(),
           "sample": f"{n} particles (strided) x {turns} turns of the same ring, "
                     f"{pet:.3e} PET in {dt:.2f} s; oracle/oracle.c, OpenMP over particles"}
    # one host thread on the first 1,024 particles of the sample, as many
    # turns as take about a quarter of a second
    orc.set_num_threads(1)
    try:
        probe = sample[:, :1024].copy()
        t = time.perf_counter()
        orc.track_until(lat, probe, 1)
        turns1 = max(1, min(1000, int(0.25 / max(time.perf_counter() - t, 1e-4))))
        one = sample[:, :1024].copy()
        t = time.perf_counter()
        orc.track_until(lat, one, turns1)
        dt1 = time.perf_counter() - t
    finally:
        orc.set_num_threads(cores)
    alive1 = sample[20, :1024].view(np.int64) == 1
    st = one[20].view(np.int64)
    pet1 = int((alive1 * one[19].view(np.int64) * n_elem).sum() +
               ((alive1 & (st == 0)) * (one[18].view(np.int64) + 1)).sum())
    out["single_thread"] = {"value": pet1 / dt1, "cores": 1,
                            "sample": f"{one.shape[1]} particles x {turns1} turns, {pet1:.3e} "
                                      f"PET in {dt1:.2f} s"}
    return out


# ------------------------------------------------------------------- e2e
def e2e_measure(ring, parts, steps, warmup, mode, threads, blocks_per_sm):
    """Through the C ABI with host buffers (TrackJob): push, track one turn,
    collect -- per step."""
    import ctypes as C

    from sixtracklib_gb300 import ParticlesSet, _native

    lib = _native.load()
    ps = ParticlesSet()
    p = ps.Particles(num_particles=parts.num_particles)
    p.set_block(parts.block)
    img_p = ps.cbuffer.to_image()
    img_e = ring.cbuffer.to_image()
    pb = lib.st_Buffer_new_on_data(img_p.ctypes.data, img_p.nbytes)
    eb = lib.st_Buffer_new_on_data(img_e.ctypes.data, img_e.nbytes)
    idx = (C.c_uint64 * 1)(0)
    job = lib.st_TrackJob_new_detailed(b"cuda", pb, 1, idx, eb, None, 0,
                                       f"mode={mode} threads_per_block={threads} "
                                       f"blocks_per_sm={blocks_per_sm}".encode())
    if not job:
        raise RuntimeError(_native.last_error())
    n_elem = len(ring)

    def alive_turns():
        sp = lib.st_Particles_buffer_get_particles(pb, 0)
        arr = C.cast(sp, C.POINTER(C.c_uint64))
        n = int(arr[0])
        col = lambda c: np.ctypeslib.as_array(  # noqa: E731
            C.cast(arr[1 + c], C.POINTER(C.c_int64)), shape=(n,)).copy()
        return col(18), col(19), col(20)  # at_element, at_turn, state

    turn = 0
    for _ in range(warmup):
        turn += 1
        lib.st_TrackJob_push_particles(job)
        lib.st_TrackJob_track_until(job, turn)
        lib.st_TrackJob_collect_particles(job)
    e0, t0, s0 = alive_turns()
    t = time.perf_counter()
    for _ in range(steps):
        turn += 1
        lib.st_TrackJob_push_particles(job)
        st = lib.st_TrackJob_track_until(job, turn)
        lib.st_TrackJob_collect_particles(job)
        if st != 0:
            raise RuntimeError(f"track status {st}: {_native.last_error()}")
    dt = time.perf_counter() - t
    e1, t1, s1 = alive_turns()
    alive0 = s0 == 1
    pet = int(((t1 - t0) * alive0).sum() * n_elem + ((alive0 & (s1 == 0)) * (e1 - e0 + 1)).sum())
    lib.st_TrackJob_delete(job)
    lib.st_Buffer_delete(pb)
    lib.st_Buffer_delete(eb)
    nbytes = parts.num_particles * 21 * 8
    return {"value": pet / dt, "unit": METRIC, "h2d_bytes_per_step": nbytes,
            "d2h_bytes_per_step": nbytes, "ms_per_step": dt / steps * 1e3}


def _build_variant(spec):
    from sixtracklib_gb300 import lattices

    seed, n_elem, _, _ = spec
    return lattices.variant_ring(seed, n_elem).cbuffer.to_image()


def build_variants(n_variants):
    """Lattice images of the batched workload, built in a spawned pool (the
    pure-Python lattice construction is the slow part)."""
    import multiprocessing as mp

    from sixtracklib_gb300 import lattices

    specs = lattices.batch_specs(n_variants=n_variants)
    with mp.get_context("spawn").Pool(min(16, os.cpu_count() or 1)) as pool:
        images = pool.map(_build_variant, specs)
    return specs, images


def per_variant_plain(dev, trk, cols, n_elem, threads=128):
    """One plain one-turn launch per variant, each timed alone with CUDA
    events: its particles, grid, time and PET/s, against which the batched
    kernel's gain is read (a variant whose grid cannot fill the GPU runs at a
    fraction of the full-GPU rate)."""
    import torch

    props = torch.cuda.get_device_properties(dev)
    stream = torch.cuda.current_stream(dev)
    rows = []
    for t, c, ne in zip(trk, cols, n_elem):
        work = c.clone()
        t.launch_until(work, 1)  # warm-up turn
        before = work.clone()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize(dev)
        a.record(stream)
        t.launch_until(work, 2)
        b.record(stream)
        torch.cuda.synchronize(dev)
        sec = a.elapsed_time(b) / 1e3
        live = int((before[20] == 1).sum())
        blocks = (live + threads - 1) // threads
        rows.append({"particles": int(c.shape[1]), "elements": int(ne), "blocks": blocks,
                     "sm_fill": min(1.0, blocks / props.multi_processor_count),
                     "ms": sec * 1e3, "value": pet_between(before, work, ne) / sec})
    return rows


def batched_measure(dev, mode, specs, images, turns=20, trial_turns=8, detail=False,
                    tune=True):
    """The batched workload over `turns` turns (after one warm-up turn): one
    tracking call per variant (plain) against one captured graph of the
    persistent batch kernel, with the launch shape autotuned first (turns
    per launch up to `trial_turns` compete)."""
    import torch

    from sixtracklib_gb300 import lattices
    from sixtracklib_gb300.batch import BatchTracker
    from sixtracklib_gb300.device import DeviceTracker

    stream = torch.cuda.current_stream(dev)
    trk = [DeviceTracker(img, config=f"mode={mode}") for img in images]
    cols = [torch.from_numpy(lattices.gaussian_particles(n, seed=ps).block.copy()
                             .view(np.int64)).to(dev) for _, _, n, ps in specs]
    n_elem = [t.num_elements for t in trk]

    def ev():
        return torch.cuda.Event(enable_timing=True)

    def pet(before, after):
        return sum(pet_between(b, a, e) for b, a, e in zip(before, after, n_elem))

    # plain: one tracking launch per variant, one variant after the other
    plain = [c.clone() for c in cols]
    for t, c in zip(trk, plain):
        t.launch_until(c, 1)  # warm-up turn
    torch.cuda.synchronize(dev)
    before = [c.clone() for c in plain]
    a, b = ev(), ev()
    a.record(stream)
    for t, c in zip(trk, plain):
        t.launch_until(c, 1 + turns)
    b.record(stream)
    torch.cuda.synchronize(dev)
    t_plain = a.elapsed_time(b) / 1e3
    pet_plain = pet(before, plain)

    work = [c.clone() for c in cols]
    bt = BatchTracker(trk)
    bt.set_particles(work)
    t0 = time.time()
    tune_ms = bt.autotune(sample_fraction=1 / 64, trial_turns=trial_turns) if tune else None
    tune_s = time.time() - t0
    assert bt.track_until(0, 1) == 0, "batch status"  # warm-up turn, as the plain arm's
    bt.capture(turns)
    before = [c.clone() for c in work]
    bt.set_turn(1)
    torch.cuda.synchronize(dev)
    a, b = ev(), ev()
    a.record(stream)
    bt.replay()
    b.record(stream)
    torch.cuda.synchronize(dev)
    t_batch = a.elapsed_time(b) / 1e3
    assert bt.status() == 0, "batch status"
    pet_batch = pet(before, work)
    identical = all(torch.equal(x, y) for x, y in zip(work, plain))
    return {
        "workload": f"{len(specs)} lattice variants, element count ~ U(500, 20000), particle "
                    f"count ~ log-uniform(1024, 262144), Gaussian 6D, FP64 {mode}",
        "particles": int(sum(c.shape[1] for c in cols)),
        "elements": int(sum(n_elem)), "turns_timed": turns,
        "plain_per_lattice": {"seconds": t_plain, "value": pet_plain / t_plain,
                              "launches": "one tracking call per variant"},
        "batched_graph": {"seconds": t_batch, "value": pet_batch / t_batch,
                          "shape": bt.shape, "autotune_s": tune_s, "autotune_trial_ms": tune_ms,
                          "autotune_trial_turns": trial_turns},
        "unit": METRIC, "speedup": t_plain / t_batch, "bit_identical": bool(identical),
        **({"per_variant_plain": per_variant_plain(dev, trk, cols, n_elem)} if detail else {}),
    }


def adjoint_measure(dev, mode, n=65536, turns=1000, every=100):
    """Forward and backward of differentiable tracking (see module doc)."""
    import torch

    from sixtracklib_gb300 import lattices
    from sixtracklib_gb300.autodiff import (DifferentiableLattice, aperture_shapes, coordinates,
                                            orbit_loss)

    ring, params = lattices.learnable_fodo_ring()
    lat = DifferentiableLattice(ring, params, f"mode={mode}")
    shapes = aperture_shapes(ring)
    cols = torch.from_numpy(lattices.gaussian_particles(n, seed=1).block.copy()
                            .view(np.int64)).to(dev)
    stream = torch.cuda.current_stream(dev)

    def ev():
        return torch.cuda.Event(enable_timing=True)

    out = {"workload": f"learnable FODO ring ({len(ring)} elements, {len(params)} strengths), "
                       f"{n} particles, {turns} turns, checkpoint every {every}",
           "loss": "mean x^2 + y^2 of the surviving particles + 1e-3 x mean smooth aperture "
                   "penalty (softplus of the normalised aperture coordinate, width 0.05)",
           "mode": mode, "particles": n, "turns": turns, "checkpoint_every": every,
           "parameters": len(params)}
    for rep in range(2):  # warm-up, then timed
        c = cols.clone()
        torch.cuda.synchronize(dev)
        a, b = ev(), ev()
        a.record(stream)
        lat.tracker.launch_until(c, turns)
        b.record(stream)
        torch.cuda.synchronize(dev)
        out["plain_forward_ms"] = a.elapsed_time(b)
    for rec in ("inverse", "recompute"):
        for rep in range(2):
            coords = coordinates(cols).clone().requires_grad_(True)
            values = torch.tensor(lat.initial_values, dtype=torch.float64, device=dev,
                                  requires_grad=True)
            torch.cuda.synchronize(dev)
            a, b, c2 = ev(), ev(), ev()
            a.record(stream)
            fin, state = lat.track(coords, values, cols, turns, checkpoint_every=every,
                                   reconstruct=rec)
            loss = orbit_loss(fin, state, shapes)
            b.record(stream)
            loss.backward()
            c2.record(stream)
            torch.cuda.synchronize(dev)
        key = "" if rec == "inverse" else "recompute_"
        out[key + "forward_ms"] = a.elapsed_time(b)
        out[key + "backward_ms"] = b.elapsed_time(c2)
        out[key + "ratio"] = out[key + "backward_ms"] / out["plain_forward_ms"]
        out[key + "grad_norm"] = float(values.grad.norm())
    out["reconstruct"] = "inverse (recompute_* keys: per-turn states recomputed)"
    return out


def bbsc_measure(n: int, turns: int, modes=("fast", "exact")) -> list:
    """Particle-element-turns/s of the beam-beam and space-charge mix
    (lattices.bb_sc_ring) with round and with elliptic strong beams: `turns`
    turns timed with CUDA events after 2 warm-up turns."""
    import torch

    from sixtracklib_gb300 import lattices
    from sixtracklib_gb300.device import DeviceTracker

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


def bbsc_bench(args, peak):
    """The beam-beam and space-charge mix (see module doc): GPU figures per
    strong-beam shape with their FP64 roofline, and the oracle on a sample of
    the same particles."""
    from sixtracklib_gb300 import lattices
    from sixtracklib_gb300.roofline import lattice_flops_per_pet

    n, turns = args.bbsc_particles, args.bbsc_turns
    gpu = bbsc_measure(n, turns, modes=(args.mode,))
    # algorithmic FP64 operations per particle-element-turn of each mix; the
    # Faddeeva function's cost depends on where a particle sits relative to
    # the strong beam: averaged over the beam's positions at the start of
    # the turn (the kicks sit together at the end of the ring, where the
    # particles are where they start)
    sample = lattices.gaussian_particles(n, seed=3)
    xs, ys = sample.x[::max(1, n // 16384)], sample.y[::max(1, n // 16384)]
    for g in gpu:
        ring = lattices.bb_sc_ring(elliptic=g["beams"] != "round")
        f = lattice_flops_per_pet(ring, xs, ys)
        achieved = g["value"] * f / 1e12
        g["roofline"] = {"bound": "fp64", "flops_per_pet": f, "achieved": achieved,
                         "peak": peak, "unit": "TFLOP/s",
                         "frac": achieved / peak if peak and peak > 0 else None,
                         "flops": "sixtracklib_gb300/roofline.py element_flops (reference "
                                  "formulas, libm calls counted as 1)"}
    out = {"workload": f"FODO ring + 4 BeamBeam6D (21 slices) + 4 BeamBeam4D + 200 "
                       f"SCQGaussProfile, {n} Gaussian protons, FP64 {args.mode}, "
                       f"{turns} turns after 2 warm-up turns",
           "unit": METRIC, "gpu": gpu}
    if not args.no_cpu:
        parts = lattices.gaussian_particles(n, seed=3)
        cpu = {}
        for g in gpu:
            ring = lattices.bb_sc_ring(elliptic=g["beams"] != "round")
            c = cpu_baseline(ring, parts, args.cpu_seconds / 2)
            cpu[g["beams"]] = c
            g["vs_cpu"] = g["value"] / c["value"]
        out["cpu_baseline"] = cpu
    return out


def tricub_bench(args, peak):
    """The TriCub workload (see module doc): PET/s with its FP64 roofline,
    the one-time cell-coefficient set-up, and the oracle on a sample."""
    import torch

    from sixtracklib_gb300 import lattices
    from sixtracklib_gb300.device import DeviceTracker
    from sixtracklib_gb300.roofline import lattice_flops_per_pet

    n, turns = args.tricub_particles, args.tricub_turns
    ring = lattices.tricub_field_ring()
    parts = lattices.gaussian_particles(n, seed=3)
    img = ring.cbuffer.to_image()
    t0 = time.perf_counter()
    trk = DeviceTracker(img, config=f"mode={args.mode} track_tricub=enabled")
    setup = time.perf_counter() - t0
    cols = torch.from_numpy(parts.block.copy().view(np.int64)).cuda()
    if trk.track_until(cols, 2) != 0:
        raise SystemExit("tricub: tracking failed")
    stream = torch.cuda.current_stream()
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    a.record(stream)
    trk.launch_until(cols, 2 + turns)
    b.record(stream)
    torch.cuda.synchronize()
    if trk.last_status() != 0:
        raise SystemExit("tricub: tracking failed")
    sec = a.elapsed_time(b) / 1e3
    alive = int((cols[20] == 1).sum())
    value = alive * len(ring) * turns / sec
    f = lattice_flops_per_pet(ring)
    achieved = value * f / 1e12
    out = {"workload": f"FODO ring + 64 TriCub kicks on one 100 x 100 x 50 map ({len(ring)} "
                       f"elements), {n} Gaussian protons, FP64 {args.mode}, {turns} turns "
                       f"after 2 warm-up turns",
           "unit": METRIC, "value": value, "ms_per_turn": sec / turns * 1e3, "alive": alive,
           "setup_s": setup,
           "roofline": {"bound": "fp64", "flops_per_pet": f, "achieved": achieved,
                        "peak": peak, "unit": "TFLOP/s",
                        "frac": achieved / peak if peak and peak > 0 else None,
                        "flops": "sixtracklib_gb300/roofline.py (TriCub: Horner form from "
                                 "per-cell coefficients)"}}
    if not args.no_cpu:
        c = cpu_baseline(ring, parts, args.cpu_seconds / 2, flags=(2, 2, 2, 2))
        out["cpu_baseline"] = c
        out["vs_cpu"] = value / c["value"]
    return out


def aggregate_over_ranks(pet, elapsed, device):
    """Whole-job figures of a weak-scaling run: PET summed over ranks, time =
    the slowest rank's (every rank tracks its own particles, no exchange)."""
    import torch
    import torch.distributed as dist

    tt = torch.tensor([float(elapsed)], device=device, dtype=torch.float64)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    pp = torch.tensor([float(pet)], device=device, dtype=torch.float64)
    dist.all_reduce(pp)
    return float(pp.item()), float(tt.item())


def shard_range(n_total, rank, world):
    """Contiguous particle range of `rank` when n_total particles are split
    over `world` ranks (used when a fixed beam is divided, strong scaling)."""
    base, extra = divmod(n_total, world)
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


# ------------------------------------------------------------------- main
def run_reference(args):
    rank, world, local = dist_env()
    if rank != 0:
        return
    from sixtracklib_gb300 import lattices

    from oracle.pyoracle import Oracle

    ring = lattices.synthetic_ring()
    parts = lattices.polar_grid_particles(args.particles)
    orc = Oracle()
    lat = ring.cbuffer.to_image()
    n_elem = len(ring)
    n = 8192
    stride = max(1, parts.num_particles // n)
    sample = parts.block[:, ::stride][:, :n].copy()
    b = sample.copy()
    turn = 0
    for _ in range(args.warmup):
        turn += 1
        orc.track_until(lat, b, turn)
    before = b.copy()
    t = time.perf_counter()
    for _ in range(args.steps):
        turn += 1
        orc.track_until(lat, b, turn)
    dt = time.perf_counter() - t
    s0 = before[20].view(np.int64) == 1
    pet = int((((b[19].view(np.int64) - before[19].view(np.int64)) * s0).sum()) * n_elem
              + ((s0 & (b[20].view(np.int64) == 0)) * (b[18].view(np.int64) + 1)).sum())
    val = pet / dt
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    line = {
        "impl": "reference", "metric": METRIC, "value": val, "unit": METRIC,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": dt / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "sample_particles": n, "lattice_elements": n_elem},
        "cpu_baseline": {"value": val, "unit": METRIC, "cores": cores, "kind": "port",
                         "cpu": host_cpu_model(),
                         "sample": f"{n} of the {args.particles} particles (strided), one turn "
                                   "per step; the CPU restatement of the reference loop "
                                   "(oracle/oracle.c, pinned bit for bit to the reference's "
                                   "own build) -- the reference's sources, from which its "
                                   "build is made, are not on the GPU host"},
        "e2e": {"value": val, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_ours(args):
    rank, world, local = dist_env()
    variants = None
    if not args.no_batched and rank == 0:
        variants = build_variants(args.batch_variants)  # before any CUDA call
    import torch

    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local if world > 1 else 0)
    torch.cuda.set_device(dev)

    from sixtracklib_gb300 import _native
    from sixtracklib_gb300.device import DeviceTracker
    from sixtracklib_gb300.roofline import lattice_flops_per_element

    lib = _native.load()
    ring, parts = make_workload(args.particles)
    n_elem = len(ring)
    cfg = (f"mode={args.mode} threads_per_block={args.threads} "
           f"blocks_per_sm={args.blocks_per_sm}")
    trk = DeviceTracker(ring.cbuffer, config=cfg)
    cols = torch.from_numpy(parts.block.copy().view(np.int64)).to(dev)
    stream = torch.cuda.current_stream(dev)

    turn = 0
    for _ in range(args.warmup):
        turn += 1
        trk.launch_until(cols, turn)
    assert trk.last_status() == 0, _native.last_error()
    before = cols[17:].clone()
    launches0 = lib.st_engine_kernel_launches()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(args.steps)]
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize(dev)
    with ClockSampler(dev.index or 0) as clocks:
        t_start = torch.cuda.Event(enable_timing=True)
        t_end = torch.cuda.Event(enable_timing=True)
        t_start.record(stream)
        for k in range(args.steps):
            turn += 1
            evs[k][0].record(stream)
            trk.launch_until(cols, turn)
            evs[k][1].record(stream)
        t_end.record(stream)
        torch.cuda.synchronize(dev)
    if world > 1:
        torch.distributed.barrier()
    status = trk.last_status()
    assert status == 0, f"track status {status}: {_native.last_error()}"
    launches = lib.st_engine_kernel_launches() - launches0
    elapsed = t_start.elapsed_time(t_end) / 1e3
    kernel_s = [a.elapsed_time(b) / 1e3 for a, b in evs]
    after = cols[17:]
    b4 = torch.zeros(21, before.shape[1], dtype=torch.int64, device=dev)
    b4[17:] = before
    af = torch.zeros_like(b4)
    af[17:] = after
    pet = pet_between(b4, af, n_elem)
    pet_total, t_max = aggregate_over_ranks(pet, elapsed, dev) if world > 1 else (pet, elapsed)
    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return
    value = pet_total / t_max
    flops_per_pet = lattice_flops_per_element(ring.cbuffer)
    pet_per_launch = pet / args.steps
    avg_launch = float(np.mean(kernel_s))
    achieved = pet_per_launch * flops_per_pet / avg_launch / 1e12
    peak = lib.st_engine_measure_fp64_peak(dev.index or 0)
    hbm_peak = None
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            hbm_peak = json.load(f).get("hbm_gbs")
    except Exception:
        pass
    alg_bytes = args.particles * 21 * 8 + args.particles * 13 * 8  # read all, write mutable
    line = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_max / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded lattice and particles)",
        "config": {"workload": (WORKLOAD if args.particles == 1_000_000 else
                                WORKLOAD.replace("1M particles", f"{args.particles} particles")),
                   "particles_per_gpu": args.particles,
                   "lattice_elements": n_elem, "turns_per_step": 1, "mode": args.mode,
                   "threads_per_block": args.threads, "blocks_per_sm": args.blocks_per_sm,
                   "l2": "inputs larger than L2: 168 MB particle columns per GPU",
                   "parallelism": f"particles sharded, {world} independent GPU(s)"},
        "gpu_launches": int(launches),
        "roofline": {"bound": "fp64", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak if peak and peak > 0 else None,
                     "traffic": (TRACK_TRAFFIC_BYTES if (args.particles, args.mode, args.threads,
                                                        args.blocks_per_sm) ==
                                 (1_000_000, "fast", 128, 2) else None),
                     "traffic_unit": "bytes per launch (ncu capture of this configuration)",
                     "peak_source": "measured in-process: dense DFMA loop (csrc/probe.cu), "
                                    "FMA = 2 flops",
                     "flops_per_pet": flops_per_pet, "launch_ms": avg_launch * 1e3,
                     "hbm_achieved_gbs": alg_bytes / avg_launch / 1e9,
                     "hbm_peak_gbs": hbm_peak},
        "clocks": clocks.summary(),
    }
    if not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(ring, parts, args.cpu_seconds)
    if variants is not None:
        try:
            line["batched"] = batched_measure(dev, args.mode, *variants,
                                              turns=args.batched_turns,
                                              detail=args.batched_detail,
                                              tune=not args.batched_no_tune)
        except Exception as exc:  # report, do not hide
            line["batched"] = {"error": str(exc)}
    if not args.no_adjoint:
        try:
            line["adjoint"] = adjoint_measure(dev, args.mode, n=args.adjoint_particles,
                                              turns=args.adjoint_turns)
        except Exception as exc:  # report, do not hide
            line["adjoint"] = {"error": str(exc)}
    if not args.no_bbsc:
        try:
            line["beam_beam_space_charge"] = bbsc_bench(args, peak)
        except Exception as exc:  # report, do not hide
            line["beam_beam_space_charge"] = {"error": str(exc)}
    if not args.no_tricub:
        try:
            line["tricub"] = tricub_bench(args, peak)
        except Exception as exc:  # report, do not hide
            line["tricub"] = {"error": str(exc)}
    if not args.no_e2e:
        try:
            line["e2e"] = e2e_measure(ring, parts, max(2, args.steps // 2), 1, args.mode,
                                      args.threads, args.blocks_per_sm)
        except Exception as exc:  # report, do not hide
            line["e2e"] = {"error": str(exc)}
    print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
