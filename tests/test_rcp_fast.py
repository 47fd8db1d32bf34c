"""The fast arithmetic policy's reciprocal (maps.cuh rcp_fast: the
hardware's reciprocal estimate refined by one third-order step): within one
ulp of 1 / x over [2^-1000, 2^1001) on the GPU, and the IEEE division
outside that range (zero, subnormals, huge values, inf, NaN)."""

import numpy as np
import pytest


def ulp_err(got, x):
    """|got - 1/x| in ulps of 1/x, 1/x in extended precision where the host
    has it."""
    ref = 1.0 / x.astype(np.longdouble)
    spacing = np.spacing(np.abs(ref.astype(np.float64)))
    return np.abs(got.astype(np.longdouble) - ref).astype(np.float64) / spacing


@pytest.mark.gpu
def test_within_one_ulp_of_the_reciprocal():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("GPU tests need a CUDA device")
    from sixtracklib_gb300 import _native

    lib = _native.load()
    rng = np.random.default_rng(23)
    mant = rng.uniform(1.0, 2.0, 3_000_000)
    x = np.concatenate([
        mant[:1_000_000] * 2.0 ** rng.integers(-1000, 1001, 1_000_000),
        mant[1_000_000:2_000_000],                        # one binade, every mantissa region
        -mant[2_000_000:] * 2.0 ** rng.integers(-80, 80, 1_000_000),
        np.nextafter(1.0, 2.0) + np.arange(1000) * 2.0 ** -52,
        2.0 ** np.arange(-1000, 1001).astype(np.float64),
    ])
    specials = np.array([0.0, -0.0, 5e-324, -5e-324, 2.0 ** -1001, 2.0 ** -1022, 2.0 ** 1001,
                         -2.0 ** 1001, 1.7976931348623157e308, np.inf, -np.inf, np.nan])
    dx = torch.from_numpy(np.concatenate([x, specials])).cuda()
    dy = torch.empty_like(dx)
    assert lib.st_engine_rcp_fast(dx.data_ptr(), dy.data_ptr(), dx.numel(), None) == 0
    torch.cuda.synchronize()
    y = dy.cpu().numpy()
    ieee = (1.0 / dx).cpu().numpy()
    err = ulp_err(y[:x.size], x)
    print(f"rcp_fast max {err.max():.3f} ulp, equal to the IEEE reciprocal at "
          f"{(y[:x.size] == ieee[:x.size]).mean():.4f} of the points")
    assert err.max() <= 1.0
    # outside the refined range: the IEEE division
    assert np.array_equal(y[x.size:], ieee[x.size:], equal_nan=True)
