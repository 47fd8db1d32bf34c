"""The reference's own CUDA tracking kernel on the GPU -- TEST
INFRASTRUCTURE ONLY (a second GPU baseline and a parity pin for the engine).

``oracle/build_ref_cuda.sh`` compiles ``sixtracklib/cuda/kernels/
track_particles.cu`` and ``managed_buffer_remap.cu`` from the reference
sources, for sm_103a with the reference's release flags (``-fmad=false``),
into ``oracle/_ref/ref_track_sm103a.cubin``.  This module loads that cubin
through the CUDA driver API and launches it the way the reference's CUDA
TrackJob does (``cuda/wrappers/controller_wrappers.cu:47``,
``cuda/wrappers/track_job_wrappers.cu:68``, ``cuda/control/
kernel_config.cpp:186-217``):

* each buffer is a CObjects image copied to the device as is and remapped
  there by ``NS(ManagedBuffer_remap_cuda)`` with one thread;
* ``NS(Track_particles_until_turn_cuda)`` / ``NS(Track_particles_line_cuda)``
  run with 128 threads per block (``DEFAULT_TRACK_THREADS_PER_BLOCK``,
  ``cuda/track_job.hpp:75``) and ceil(particles / 128) blocks, on the
  particle set's image and the lattice image, slot size 8.

Device memory comes from PyTorch; the kernels run on PyTorch's current
stream.  Nothing here is part of the engine.
"""

from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
CUBIN = os.path.join(HERE, "_ref", "ref_track_sm103a.cubin")
SLOT_SIZE = 8
THREADS_PER_BLOCK = 128

_cu = None


def available() -> bool:
    return os.path.exists(CUBIN)


def _driver():
    global _cu
    if _cu is None:
        _cu = C.CDLL("libcuda.so.1")
    return _cu


def _check(res: int, what: str) -> None:
    if res != 0:
        name = C.c_char_p()
        _driver().cuGetErrorName(int(res), C.byref(name))
        raise RuntimeError(f"{what}: CUDA driver error {res} "
                           f"({name.value.decode() if name.value else '?'})")


class RefCudaKernels:
    """The reference's remap, until-turn and line kernels, loaded once."""

    def __init__(self, torch, cubin: str = CUBIN):
        if not os.path.exists(cubin):
            raise FileNotFoundError(f"{cubin} is missing: run oracle/build_ref_cuda.sh "
                                    f"where the reference sources are present")
        self.torch = torch
        torch.cuda.init()
        torch.empty(1, device="cuda")  # the primary context exists and is current
        cu = _driver()
        ctx = C.c_void_p()
        _check(cu.cuCtxGetCurrent(C.byref(ctx)), "cuCtxGetCurrent")
        if not ctx.value:
            dev = C.c_int()
            _check(cu.cuDeviceGet(C.byref(dev), torch.cuda.current_device()), "cuDeviceGet")
            _check(cu.cuDevicePrimaryCtxRetain(C.byref(ctx), dev), "cuDevicePrimaryCtxRetain")
            _check(cu.cuCtxSetCurrent(ctx), "cuCtxSetCurrent")
        self.module = C.c_void_p()
        _check(cu.cuModuleLoad(C.byref(self.module), cubin.encode()), "cuModuleLoad")
        self.fn = {}
        for name in ("st_ManagedBuffer_remap_cuda", "st_Track_particles_until_turn_cuda",
                     "st_Track_particles_line_cuda"):
            f = C.c_void_p()
            _check(cu.cuModuleGetFunction(C.byref(f), self.module, name.encode()), name)
            self.fn[name] = f

    def _launch(self, name, blocks, threads, args):
        vals = [C.c_uint64(int(a)) if not isinstance(a, C._SimpleCData) else a for a in args]
        ptrs = (C.c_void_p * len(vals))(*[C.cast(C.byref(v), C.c_void_p) for v in vals])
        stream = C.c_void_p(self.torch.cuda.current_stream().cuda_stream)
        _check(_driver().cuLaunchKernel(self.fn[name], C.c_uint(blocks), C.c_uint(1), C.c_uint(1),
                                        C.c_uint(threads), C.c_uint(1), C.c_uint(1), C.c_uint(0),
                                        stream, ptrs, None), name)

    def to_device(self, image: np.ndarray):
        """A device copy of a CObjects image, remapped on the device."""
        img = np.ascontiguousarray(image).view(np.uint8)
        d = self.torch.from_numpy(img.copy()).cuda()
        self._launch("st_ManagedBuffer_remap_cuda", 1, 1, [d.data_ptr(), SLOT_SIZE])
        return d

    def track_until(self, d_particles, num_particles, d_lattice, until_turn, pset_index=0,
                    threads=THREADS_PER_BLOCK):
        blocks = max(1, -(-int(num_particles) // threads))
        self._launch("st_Track_particles_until_turn_cuda", blocks, threads,
                     [d_particles.data_ptr(), pset_index, d_lattice.data_ptr(), until_turn,
                      SLOT_SIZE])

    def track_line(self, d_particles, num_particles, d_lattice, begin, end, finish_turn,
                   pset_index=0, threads=THREADS_PER_BLOCK):
        blocks = max(1, -(-int(num_particles) // threads))
        self._launch("st_Track_particles_line_cuda", blocks, threads,
                     [d_particles.data_ptr(), pset_index, d_lattice.data_ptr(), begin, end,
                      C.c_bool(bool(finish_turn)), SLOT_SIZE])


def particles_image(block: np.ndarray) -> np.ndarray:
    """The CObjects image of one particle set holding a 21 x n column block."""
    from sixtracklib_gb300.particles import ParticlesSet

    ps = ParticlesSet()
    ps.Particles(num_particles=block.shape[1]).set_block(block)
    return ps.cbuffer.to_image()


def particles_block(d_particles) -> np.ndarray:
    """The 21 x n column block of particle set 0 of a device particle image."""
    from sixtracklib_gb300.cbuffer import CBuffer
    from sixtracklib_gb300.particles import Particles, TYPE_PARTICLE

    img = d_particles.cpu().numpy().view(np.uint64)
    cb = CBuffer.from_image(img)
    cb.typeids[TYPE_PARTICLE] = Particles
    return cb.get_object(0).block.copy()


def track_until(torch, lattice_image, block, until_turn):
    """Track a 21 x n column block with the reference's CUDA kernel; returns
    the tracked block."""
    k = RefCudaKernels(torch)
    lat = k.to_device(lattice_image)
    parts = k.to_device(particles_image(block))
    k.track_until(parts, block.shape[1], lat, until_turn)
    torch.cuda.synchronize()
    return particles_block(parts)


def _pet(before: np.ndarray, after: np.ndarray, n_elem: int) -> int:
    """Particle-element-turns between two column blocks (a particle lost at
    element k of its last turn counts k + 1 there)."""
    alive0 = before[20].view(np.int64) == 1
    turns = after[19].view(np.int64) - before[19].view(np.int64)
    lost = alive0 & (after[20].view(np.int64) == 0)
    e0, e1 = before[18].view(np.int64), after[18].view(np.int64)
    return int(np.where(alive0, turns * n_elem, 0).sum() + np.where(lost, e1 - e0 + 1, 0).sum())


def main(argv=None):
    """Time the reference's CUDA kernel on the synthetic 20,000-element ring
    and the polar-grid protons (the engine's benchmark workload), or on the
    beam-beam and space-charge mix (round or elliptic strong beams, Gaussian
    protons): one warm-up turn, then `turns` turns in one launch timed with
    CUDA events; prints one JSON line."""
    import argparse
    import json

    import torch

    from sixtracklib_gb300 import lattices

    ap = argparse.ArgumentParser()
    ap.add_argument("--particles", type=int, default=1_000_000)
    ap.add_argument("--turns", type=int, default=2)
    ap.add_argument("--workload", default="synthetic",
                    choices=["synthetic", "bbsc", "bbsc_elliptic"])
    args = ap.parse_args(argv)
    if args.workload == "synthetic":
        ring = lattices.synthetic_ring()
        parts = lattices.polar_grid_particles(args.particles)
        name = f"synthetic 20k-element ring, {args.particles} particles polar grid"
    else:
        elliptic = args.workload == "bbsc_elliptic"
        ring = lattices.bb_sc_ring(elliptic=elliptic)
        parts = lattices.gaussian_particles(args.particles, seed=3)
        name = (f"FODO ring + 4 BeamBeam6D (21 slices) + 4 BeamBeam4D + 200 SCQGaussProfile, "
                f"{'elliptic' if elliptic else 'round'} strong beams, {args.particles} "
                f"Gaussian protons")
    k = RefCudaKernels(torch)
    d_lat = k.to_device(ring.cbuffer.to_image())
    d_p = k.to_device(particles_image(parts.block))
    n = parts.block.shape[1]
    k.track_until(d_p, n, d_lat, 1)
    torch.cuda.synchronize()
    before = particles_block(d_p)
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    start.record()
    k.track_until(d_p, n, d_lat, 1 + args.turns)
    stop.record()
    torch.cuda.synchronize()
    ms = start.elapsed_time(stop)
    after = particles_block(d_p)
    pet = _pet(before, after, len(ring))
    print(json.dumps({
        "kernel": "st_Track_particles_until_turn_cuda (reference, sm_103a, -fmad=false)",
        "workload": f"{name}, {args.turns} turns after 1 warm-up turn, "
                    f"{THREADS_PER_BLOCK} threads per block",
        "ms": ms, "pet": pet, "value": pet / (ms * 1e-3),
        "unit": "particle-element-turns/s"}))


if __name__ == "__main__":
    main()
