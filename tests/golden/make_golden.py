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
3. Outputs of the reference's own tracking code on the reference's shipped
   machine descriptions (`lhc_no_bb`, `beambeam`): ref_shipped_<name>.npz
   (`python tests/golden/make_golden.py --shipped` makes only these).
4. Gradients of 1,000-turn differentiable tracking from the dual-number
   oracle: adjoint_fodo_1000.npz (`--adjoint` makes only this one).
5. The shipped lattices' 6D beam-beam elements: lab-frame parameters and
   the stored payloads, bb6d_shipped.npz (`--bb6d`).
6. The shipped pysixtrack lines of `bbsimple` and `beambeam` as gzipped
   JSON, line_<name>.json.gz (`--lines`).
7. The TriCub map and the map feature flags (`--tricub`): the reference's
   TriCub known-answer kicks (tests/testdata/tricub/precomputed_kicks.txt,
   read as text) with their seed, tricub_kicks.npz; the reference's builds
   with other feature flags (oracle/_ref/libstref_flags_{a,b}.so, TriCub
   enabled in `a`) tracking tests/tricub_cases.py's lattices,
   ref_tricub.npz and ref_flags.npz.
"""

from __future__ import annotations

import hashlib
import os
import sys
from math import factorial

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


SHIPPED_SAMPLE = 1024
SHIPPED_TURNS = (1, 1000)


def shipped_lattices():
    """The reference's shipped machine descriptions (tests/testdata):
    `lhc_no_bb` (18,657 elements: Drift, Multipole, Cavity, XYShift,
    SRotation) and `beambeam` (10,866: Drift, Multipole, Cavity, 72
    BeamBeam4D, 2 pysixtrack-initialised BeamBeam6D).  Their particle dumps
    are not shipped (the generator needs pysixtrack / sixtracktools), so a
    seeded 1,024-proton sample at 6.5 TeV (the energy of both SixTrack inputs,
    fort.3) is tracked 1 and 1,000 turns by the reference build and stored:
    ref_shipped_<name>.npz holds the lattice image, the initial block and the
    final block and status after each turn count."""
    ref = Oracle.reference(omp=True)
    if ref is None:
        raise SystemExit("reference build not available (REF_ROOT)")
    for seed, name in ((21, "lhc_no_bb"), (22, "beambeam")):
        cb = CBuffer.fromfile(os.path.join(TD, name, "beam_elements.bin"))
        img = cb.to_image()
        p = lattices.gaussian_particles(SHIPPED_SAMPLE, seed=seed, sx=1e-4, spx=1e-6, sy=1e-4,
                                        spy=1e-6, sz=0.02, sdelta=1e-4, p0c=6.5e12)
        init = p.block.copy()
        arrays = dict(lattice=img, initial=init, lattice_sha256=np.array(image_hash(img)))
        for turns in SHIPPED_TURNS:
            fin = init.copy()
            st = ref.track_until(img, fin, turns)
            arrays[f"final_{turns}"] = fin
            arrays[f"status_{turns}"] = np.int64(st)
            lost = int((fin[20].view(np.int64) == 0).sum())
            print(f"ref_shipped_{name}: {turns} turns, status {st}, lost {lost}")
        np.savez_compressed(os.path.join(HERE, f"ref_shipped_{name}.npz"), **arrays)


ADJ_PARTICLES = 256
ADJ_TURNS = 1000
ADJ_EDGE = 8  # particles started near the LimitRect edge (lost within the run)
SIGMA = np.array([1e-3, 1e-5, 1e-3, 1e-5, 0.05, 1e-4])


def adjoint_beam():
    """The 256-particle beam of the differentiable-tracking fixture: the
    Gaussian beam of the learnable FODO ring with ADJ_EDGE particles started
    at x in [0.013, 0.019] m, close to the +-0.02 m LimitRect."""
    from sixtracklib_gb300.particles import COL

    blk = lattices.gaussian_particles(ADJ_PARTICLES, seed=41).block.copy()
    blk.view(np.float64)[COL["x"], :ADJ_EDGE] = np.linspace(0.013, 0.019, ADJ_EDGE)
    return blk


def adjoint_fixture():
    """Gradients of 1,000-turn tracking on the learnable FODO ring (64 quad
    strengths, 16 sextupoles; the differentiable-tracking workload) from the
    dual-number oracle (oracle/dual.py, pinned to the C oracle and to finite
    differences on the CPU), for two objectives: a random linear functional
    of the final coordinates (every Jacobian entry) and the workload's
    objective autodiff.orbit_loss (mean x^2 + y^2 of the survivors plus the
    smooth aperture penalty).  The dual pass takes a few minutes, too long
    for a GPU test, so its results are stored: adjoint_fodo_1000.npz."""
    import torch

    from oracle import dual
    from sixtracklib_gb300.autodiff import aperture_shapes, orbit_loss

    ring, params = lattices.learnable_fodo_ring()
    blk = adjoint_beam()
    kinds = [(int(p[0]), -1 if p[1] == "voltage" else 2 * int(p[2]) + (p[1] == "ksl"))
             for p in params]
    scale = np.array([1.0 if p[1] == "voltage" else 1.0 / factorial(int(p[2])) for p in params])
    vals, ders, st, at, ae = dual.track_until(ring, blk.copy(), ADJ_TURNS, params=kinds)
    w = np.random.default_rng(42).normal(size=(6, ADJ_PARTICLES)) / SIGMA[:, None]
    out = torch.from_numpy(vals.copy()).requires_grad_(True)
    loss = orbit_loss(out, torch.from_numpy(st.astype(np.int64)), aperture_shapes(ring))
    loss.backward()
    dl = out.grad.numpy()
    arrays = dict(initial=blk, values=vals, state=st.astype(np.int64),
                  at_turn=np.asarray(at, np.int64), at_element=np.asarray(ae, np.int64),
                  weights=w, turns=np.int64(ADJ_TURNS),
                  linear_grad_coords=np.einsum("rn,crn->cn", w, ders[:6]),
                  linear_grad_params=np.einsum("rn,jrn->j", w, ders[6:]) * scale,
                  loss=np.float64(loss.item()),
                  loss_grad_coords=np.einsum("rn,crn->cn", dl, ders[:6]),
                  loss_grad_params=np.einsum("rn,jrn->j", dl, ders[6:]) * scale)
    np.savez_compressed(os.path.join(HERE, "adjoint_fodo_1000.npz"), **arrays)
    print(f"adjoint_fodo_1000: lost {int((st == 0).sum())}/{ADJ_PARTICLES}, "
          f"loss {loss.item():.6e}")


BB6D_KEYS = ("q_part", "N_part_tot", "sigmaz", "N_slices", "min_sigma_diff",
             "threshold_singular", "phi", "alpha", "Sig_11_0", "Sig_12_0", "Sig_13_0",
             "Sig_14_0", "Sig_22_0", "Sig_23_0", "Sig_24_0", "Sig_33_0", "Sig_34_0",
             "Sig_44_0", "delta_x", "delta_y", "x_CO", "px_CO", "y_CO", "py_CO", "sigma_CO",
             "delta_CO", "Dx_sub", "Dpx_sub", "Dy_sub", "Dpy_sub", "Dsigma_sub", "Ddelta_sub",
             "enabled")


def bb6d_fixture():
    """The 6D beam-beam elements of the reference's shipped `bbsimple` and
    `beambeam` lattices, twice: the strong-beam parameters in the lab frame
    as the pysixtrack line of the same test data holds them (line.pkl, read
    as data: its objects are restored into plain stand-in classes, nothing
    of pysixtrack is imported), and the payload words pysixtrack's
    initialisation wrote into beam_elements.bin.  bb6d_shipped.npz:
    `<lattice>_params` (one row per element, columns BB6D_KEYS) and
    `<lattice>_payload_<k>`."""
    import pickle

    class _Stub:
        def __setstate__(self, state):
            if isinstance(state, tuple):
                for part in state:
                    if isinstance(part, dict):
                        self.__dict__.update(part)
            elif isinstance(state, dict):
                self.__dict__.update(state)

    class _Reader(pickle.Unpickler):
        def find_class(self, module, name):
            if module.startswith(("pysixtrack", "sixtracktools", "__main__")):
                return type(name, (_Stub,), {})
            return super().find_class(module, name)

    arrays = {}
    for name in ("bbsimple", "beambeam"):
        with open(os.path.join(TD, name, "line.pkl"), "rb") as f:
            line = _Reader(f).load()
        rows = []
        for item in line:
            el = item[-1] if isinstance(item, tuple) else item
            if type(el).__name__ == "BeamBeam6D":
                rows.append([float(getattr(el, k)) for k in BB6D_KEYS])
        stored = [np.asarray(o.data, dtype=np.float64)
                  for o in Elements.fromfile(os.path.join(TD, name, "beam_elements.bin"))
                  .get_elements() if type(o).__name__ == "BeamBeam6D"]
        assert len(rows) == len(stored) > 0
        arrays[f"{name}_params"] = np.array(rows)
        for k, w in enumerate(stored):
            arrays[f"{name}_payload_{k}"] = w
        print(f"bb6d_shipped: {name}: {len(rows)} BeamBeam6D elements")
    np.savez_compressed(os.path.join(HERE, "bb6d_shipped.npz"), keys=np.array(BB6D_KEYS),
                        **arrays)


def lines_fixture():
    """The pysixtrack lines of the shipped `bbsimple` and `beambeam` test data
    (line.pkl, read as data into stand-in classes, nothing of pysixtrack
    imported): per element its class name and attributes, as gzipped JSON
    (line_<name>.json.gz).  The shipped beam_elements.bin were written from
    these lines by the reference's Elements.fromline."""
    import gzip
    import json
    import pickle

    class _Stub:
        def __setstate__(self, state):
            for part in (state if isinstance(state, tuple) else (state,)):
                if isinstance(part, dict):
                    self.__dict__.update(part)

    class _Reader(pickle.Unpickler):
        def find_class(self, module, name):
            if module.startswith(("pysixtrack", "sixtracktools", "__main__")):
                return type(name, (_Stub,), {})
            return super().find_class(module, name)

    for name in ("bbsimple", "beambeam"):
        with open(os.path.join(TD, name, "line.pkl"), "rb") as f:
            line = _Reader(f).load()
        out = []
        for item in line:
            el = item[-1] if isinstance(item, tuple) else item
            attrs = {k: (v.tolist() if hasattr(v, "tolist") else v)
                     for k, v in el.__dict__.items() if not k.startswith("_")}
            out.append([type(el).__name__, attrs])
        with gzip.open(os.path.join(HERE, f"line_{name}.json.gz"), "wt") as f:
            json.dump(out, f)
        print(f"line_{name}: {len(out)} elements")


def tricub_fixtures():
    """tricub_kicks.npz, ref_tricub.npz, ref_flags.npz (see the module doc)."""
    sys.path.insert(0, os.path.dirname(HERE))
    import tricub_cases as tc

    with open(os.path.join(TD, "tricub", "precomputed_kicks.txt")) as f:
        rows = [r.split() for r in f.read().strip().split("\n")]
    kicks = np.array([[float(v) for v in r] for r in rows[:-1]])
    seed = int(float(rows[-1][0]))
    np.savez_compressed(os.path.join(HERE, "tricub_kicks.npz"), kicks=kicks,
                        seed=np.int64(seed))
    print(f"tricub_kicks: {kicks.shape[0]} particles, seed {seed}")

    orc = Oracle()
    ref_a = Oracle.reference(flags="a")
    if ref_a is None:
        raise SystemExit("reference build not available (REF_ROOT)")
    # the reference reads outside its table for a particle outside the grid:
    # the oracle (which stops such a particle) runs first and must succeed
    ring = tc.tricub_ring()
    img = ring.cbuffer.to_image()
    p = tc.tricub_particles(512, 21)
    arrays = dict(lattice=img, initial=p.block.copy())
    orc.set_track_flags(*tc.FLAG_BUILDS["a"])
    for turns in (1, 20):
        chk = p.block.copy()
        if orc.track_until(img, chk, turns) != 0:
            raise SystemExit("tricub ring: a particle leaves a grid")
        fin = p.block.copy()
        arrays[f"final_{turns}"] = fin
        arrays[f"status_{turns}"] = np.int64(ref_a.track_until(img, fin, turns))
    np.savez_compressed(os.path.join(HERE, "ref_tricub.npz"), **arrays)

    lat = tc.flags_lattice()
    img = lat.cbuffer.to_image()
    p = tc.tricub_particles(64, 8)
    arrays = dict(lattice=img, initial=p.block.copy())
    for name, flags in tc.FLAG_BUILDS.items():
        ref = Oracle.reference(flags=None if name == "default" else name)
        fin = p.block.copy()
        arrays[f"until_{name}"] = fin
        arrays[f"until_status_{name}"] = np.int64(ref.track_until(img, fin, 3))
        lines, status = [], []
        for k in range(len(lat)):
            fin = p.block.copy()
            status.append(ref.track_line(img, fin, k, k + 1))
            lines.append(fin)
        arrays[f"line_{name}"] = np.stack(lines)
        arrays[f"line_status_{name}"] = np.array(status, dtype=np.int64)
    np.savez_compressed(os.path.join(HERE, "ref_flags.npz"), **arrays)
    print("ref_tricub, ref_flags written")


def main():
    if "--tricub" in sys.argv:
        tricub_fixtures()
        return
    if "--lines" in sys.argv:
        lines_fixture()
        return
    if "--bb6d" in sys.argv:
        bb6d_fixture()
        return
    if "--shipped" in sys.argv:
        shipped_lattices()
        return
    if "--adjoint" in sys.argv:
        adjoint_fixture()
        return
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
    shipped_lattices()
    adjoint_fixture()
    bb6d_fixture()
    lines_fixture()
    print("fixtures written to", HERE)


if __name__ == "__main__":
    main()
