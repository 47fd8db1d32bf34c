"""The 6D beam-beam set-up (beam_elements.bb6d_data and
gaussian_equal_charge_slices) against what the reference ships and its own
boost maps.

The reference delegates the set-up to pysixtrack (BB6D_init, called at
python/sixtracklib/beam_elements.py:496-543), which is not in its tree.
Three checks pin the own implementation:

* the shipped payloads: the 6D beam-beam elements of the `bbsimple` and
  `beambeam` test lattices, rebuilt from the lab-frame parameters of the
  pysixtrack line in the same test data (tests/golden/bb6d_shipped.npz),
  reproduce the words pysixtrack wrote into beam_elements.bin;
* the boosted slice centroids equal the reference's own
  NS(BeamBeam6D_boost) (be_beamfields.h:2101-2160) applied to the strong
  bunch's slice positions (0, 0, 0, 0, z, 0);
* the reference's boost followed by its inverse boost (be_beamfields.h:
  2162-2230) is the identity on the set-up's boost parameters.
"""

import ctypes as C
import os

import numpy as np
import pytest

from sixtracklib_gb300.beam_elements import bb6d_data, gaussian_equal_charge_slices

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _rebuild(p):
    keys = [str(k) for k in np.load(os.path.join(GOLDEN, "bb6d_shipped.npz"))["keys"]]
    v = dict(zip(keys, p))
    charge, z = gaussian_equal_charge_slices(v["N_part_tot"], v["sigmaz"], int(v["N_slices"]))
    sig = [v[f"Sig_{ij}_0"] for ij in ("11", "12", "13", "14", "22", "23", "24", "33", "34",
                                       "44")]
    return bb6d_data(
        q_part=v["q_part"], phi=v["phi"], alpha=v["alpha"], delta_x=v["delta_x"],
        delta_y=v["delta_y"], n_part_per_slice=charge, z_slices=z, sigmas=sig,
        co=[v[k] for k in ("x_CO", "px_CO", "y_CO", "py_CO", "sigma_CO", "delta_CO")],
        min_sigma_diff=v["min_sigma_diff"], threshold_singular=v["threshold_singular"],
        d_sub=[v[k] for k in ("Dx_sub", "Dpx_sub", "Dy_sub", "Dpy_sub", "Dsigma_sub",
                              "Ddelta_sub")],
        enabled=v["enabled"])


@pytest.mark.parametrize("name", ["bbsimple", "beambeam"])
def test_bb6d_setup_reproduces_shipped_payloads(name):
    d = np.load(os.path.join(GOLDEN, "bb6d_shipped.npz"))
    params = d[f"{name}_params"]
    for k, p in enumerate(params):
        stored = d[f"{name}_payload_{k}"]
        got = _rebuild(p)
        assert got.shape == stored.shape
        sw, gw = stored.view(np.uint64), got.view(np.uint64)
        # integer words (slice count, relative offsets) identical
        assert sw[18] == gw[18] and np.array_equal(sw[34:38], gw[34:38])
        # `enabled` is stored as the integer 1 by pysixtrack, as 1.0 here:
        # both are > 0, which is all the tracking map tests
        assert (stored[33] > 0) == (got[33] > 0)
        real = np.r_[0:18, 19:33, 38:stored.size]
        dev = np.abs(got[real] - stored[real])
        scale = np.maximum(np.abs(stored[real]), 1e-300)
        assert np.all((dev <= 4e-16 * scale) | (dev == 0)), (name, k, real[np.argmax(dev / scale)],
                                                               np.max(dev / scale))


def _ref_boost():
    from oracle.pyoracle import Oracle

    ref = Oracle.reference()
    if ref is None:
        pytest.skip("reference sources not available here")
    fn = ref.lib.ref_bb6d_boost
    fn.argtypes = [C.c_void_p, C.c_void_p, C.c_int]
    fn.restype = None

    def boost(b, c6, inverse=False):
        c = np.ascontiguousarray(c6, dtype=np.float64).copy()
        bb = np.ascontiguousarray(b, dtype=np.float64)
        fn(bb.ctypes.data, c.ctypes.data, int(inverse))
        return c
    return boost


@pytest.mark.parametrize("phi,alpha,n", [(0.5, 1.57, 2), (1.5e-4, 0.3, 5), (2.95e-4, 0.0, 21)])
def test_boosted_slice_centroids_match_reference_boost(phi, alpha, n):
    boost = _ref_boost()
    charge, z = gaussian_equal_charge_slices(1.15e11, 0.0755, n)
    w = bb6d_data(q_part=1.6e-19, phi=phi, alpha=alpha, delta_x=0.0, delta_y=0.0,
                  n_part_per_slice=charge, z_slices=z,
                  sigmas=(1e-10, 0, 0, 0, 1e-12, 0, 0, 1e-10, 0, 1e-12))
    b = w[1:6]
    xs, ys, ss = w[38 + n:38 + 2 * n], w[38 + 2 * n:38 + 3 * n], w[38 + 3 * n:38 + 4 * n]
    for k in range(n):
        c = boost(b, [0.0, 0.0, 0.0, 0.0, z[k], 0.0])
        np.testing.assert_allclose([xs[k], ys[k], ss[k]], [c[0], c[2], c[4]], rtol=4e-16,
                                   atol=1e-300)
        assert c[1] == 0.0 and c[3] == 0.0 and c[5] == 0.0


@pytest.mark.parametrize("phi,alpha", [(0.5, 1.57), (2.95e-4, 0.0), (1.5e-4, 0.3)])
def test_reference_boost_then_inverse_is_identity(phi, alpha):
    boost = _ref_boost()
    w = bb6d_data(q_part=1.6e-19, phi=phi, alpha=alpha, delta_x=0.0, delta_y=0.0,
                  n_part_per_slice=[1.0], z_slices=[0.0],
                  sigmas=(1e-10, 0, 0, 0, 1e-12, 0, 0, 1e-10, 0, 1e-12))
    rng = np.random.default_rng(5)
    scale = np.array([1e-3, 1e-4, 1e-3, 1e-4, 0.05, 1e-4])
    for _ in range(200):
        c0 = rng.normal(size=6) * scale
        c1 = boost(w[1:6], boost(w[1:6], c0), inverse=True)
        # the reference's inverse boost rounds at ~1e-12 of the coordinate
        # scale for a half crossing angle of 0.5 rad, ~1e-16 for 1e-4 rad
        tol = 1e-11 if phi > 0.1 else 1e-14
        assert np.all(np.abs(c1 - c0) <= tol * scale), (c0, c1)
