"""Generate the golden fixtures in tests/golden/.

Run in a checkout where the reference tree is mounted (REF_ROOT, default
/root/reference): it needs the reference's shipped test data and the
reference build (oracle/build_ref.sh -> oracle/_ref/libstref.so).  The GPU
machines have neither, so the fixtures are committed.

Two kinds of fixture:

1. Conversions of the reference's own known-answer data (tests/testdata):
   * bbsimple.npz   -- the pysixtrack element-by-element dump of the
     `bbsimple` lattice (Drift, Multipole, Cavity, BB4D, BB6D): lattice
     image (re-encoded by sixtracklib_gb300.cbuffer) and the 16 recorded
     particle states (2 particles each);
   * drift.npz / driftexact.npz -- first 200 particles of
     test_track_be_drift(exact)_data.bin: initial state, the 1000-element
     lattice, the expected state after one turn;
   * faddeeva.npz   -- 2,000 of the 10,000 (z, w(z)) points of
     test_faddeeva_errorfn_data.bin.
2. Outputs of the reference's own tracking code (oracle/_ref) on seeded
   synthetic inputs: ref_<case>.npz with the initial and final column blocks
   and, for small lattices, the lattice image.
"""

from __future__ import annotations

import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.pyoracle import EbeConfig, Oracle  # noqa: E402
from sixtracklib_gb300 import CBuffer, lattices  # noqa: E402
from sixtracklib_gb300.beam_elements import Elements  # noqa: E402
from sixtracklib_gb300.particles import Particles  # noqa: E402

REF = os.environ.get("REF_ROOT", "/root/reference")
TD = os.path.join(REF, "tests", "testdata")


def image_hash(img: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(img).tobytes()).hexdigest()


def particle_blocks(cb: CBuffer):
    out = []
    for i, o in enumerate(cb.objects):
        if o.typeid == 1:
            out.append(Particles._from_cobject(o, cb, i).block.copy())
    return out


def misc_lattice() -> Elements:
    e = Elements()
    e.DriftExact(length=1.5)
    e.RFMultipole(voltage=1e5, frequency=4e8, lag=30, knl=[1e-6, 0.002, 0.001],
                  ksl=[0, 1e-4], pn=[10, 20, 30], ps=[5, 6])
    e.DipoleEdge(r21=0.01, r43=-0.02)
    e.LimitRectEllipse(max_x=0.03, max_y=0.02, a=0.035, b=0.025)
    e.Multipole(knl=[1e-4, 0.005], ksl=[2e-4], hxl=1e-5, hyl=-2e-5, length=1.0)
    e.Drift(length=2.0)
    e.SCCoasting(number_of_particles=1e11, circumference=1000, sigma_x=1e-3,
                 sigma_y=1.5e-3, length=1.0)
    e.SRotation(angle=10)
    e.XYShift(dx=1e-4, dy=-1e-4)
    e.Cavity(voltage=1e6, frequency=2e8, lag=45)
    e.BeamMonitor(num_stores=4, start=0, skip=1, out_address=1, min_particle_id=0,
                  max_particle_id=63, is_rolling=1, is_turn_ordered=1)
    e.Multipole(knl=[0.0, -0.005, 0.05, 0.3])
    e.LimitRect(min_x=-0.05, max_x=0.05, min_y=-0.04, max_y=0.04)
    return e


def main():
    ref = Oracle.reference()
    if ref is None:
        raise SystemExit("reference build not available (REF_ROOT)")
    out = {}

    # ---- 1. reference known-answer data
    be = CBuffer.fromfile(os.path.join(TD, "bbsimple", "beam_elements.bin"))
    dump = CBuffer.fromfile(os.path.join(TD, "bbsimple", "particles_dump.bin"))
    states = np.stack(particle_blocks(dump))
    np.savez_compressed(os.path.join(HERE, "bbsimple.npz"), lattice=be.to_image(),
                        states=states)
    for name in ("drift", "driftexact"):
        cb = CBuffer.fromfile(os.path.join(TD, f"test_track_be_{name}_data.bin"))
        blocks = particle_blocks(cb)
        lat = CBuffer()
        for o in cb.objects[1:-1]:
            lat.add_raw(o)
        init = blocks[0][:, :200].copy()
        exp = blocks[1][:, :200].copy()
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), lattice=lat.to_image(),
                            initial=init, expected=exp)
    raw = np.fromfile(os.path.join(TD, "test_faddeeva_errorfn_data.bin"), dtype=np.uint64)
    n = int(raw[0])
    vals = raw[1:1 + 4 * n].view(np.float64).reshape(n, 4)
    sel = np.random.default_rng(1).choice(n, 2000, replace=False)
    np.savez_compressed(os.path.join(HERE, "faddeeva.npz"), points=vals[np.sort(sel)])

    # ---- 2. reference tracking outputs on seeded synthetic inputs
    cases = {}
    fodo = lattices.fodo_ring()
    cases["fodo"] = (fodo, lattices.gaussian_particles(256, seed=11), 50, True)
    syn = lattices.synthetic_ring()
    cases["synthetic"] = (syn, lattices.polar_grid_particles(66, seed=3), 2, False)
    cases["bbsc"] = (lattices.bb_sc_ring(), lattices.gaussian_particles(
        64, seed=7, sx=2e-5, sy=2e-5), 10, True)
    cases["bbsc_elliptic"] = (lattices.bb_sc_ring(elliptic=True), lattices.gaussian_particles(
        64, seed=8, sx=2e-5, sy=2e-5), 10, True)
    cases["misc"] = (misc_lattice(), lattices.gaussian_particles(
        64, seed=9, sx=9e-3, sy=7e-3, spx=1e-4, spy=1e-4), 6, True)
    for name, (lat, p, turns, store_lattice) in cases.items():
        img = lat.cbuffer.to_image()
        init = p.block.copy()
        fin = init.copy()
        mons = None
        if name == "misc":
            mons = [np.zeros((21, 4 * 64), dtype=np.uint64)]
        st = ref.track_until(img, fin, turns, monitors=mons)
        arrays = dict(initial=init, final=fin, turns=np.int64(turns), status=np.int64(st),
                      lattice_sha256=np.array(image_hash(img)))
        if store_lattice:
            arrays["lattice"] = img
        if mons:
            arrays["monitor0"] = mons[0]
        # line tracking: elements [3, 9) without and [0, E) with finish_turn
        line = init.copy()
        lmons = [np.zeros((21, 4 * 64), dtype=np.uint64)] if mons else None
        arrays["line_status"] = np.int64(ref.track_line(img, line, 3, min(9, len(lat)), False,
                                                        monitors=lmons))
        arrays["line_final"] = line
        # elem-by-elem over 2 turns
        if store_lattice and len(lat) < 400:
            ne = len(lat)
            nst = 16  # store the first 16 particle ids only
            cfg = EbeConfig(0, nst, ne, 2, 0, 0, 0, nst - 1, ne - 1, 1, 1)
            nrec = cfg.num_particles_to_store * ne * 2
            ebe_out = np.zeros((21, nrec), dtype=np.uint64)
            eb = init.copy()
            emons = [np.zeros((21, 4 * 64), dtype=np.uint64)] if mons else None
            arrays["ebe_status"] = np.int64(ref.track_elem_by_elem(img, eb, cfg, ebe_out, 2,
                                                                   monitors=emons))
            if emons:
                arrays["ebe_monitor0"] = emons[0]
            arrays["ebe_final"] = eb
            arrays["ebe_out"] = ebe_out
            arrays["ebe_cfg"] = np.array([getattr(cfg, f) for f, _ in EbeConfig._fields_],
                                         dtype=np.int64)
        np.savez_compressed(os.path.join(HERE, f"ref_{name}.npz"), **arrays)
        lost = int((fin[20].view(np.int64) == 0).sum())
        print(f"ref_{name}: status {st}, lost {lost}/{fin.shape[1]}")
    print("fixtures written to", HERE)


if __name__ == "__main__":
    main()
