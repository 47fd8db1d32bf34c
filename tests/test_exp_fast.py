"""The fast arithmetic policy's exponential (maps.cuh exp_fast, a
table-driven e^x after P. T. P. Tang, ACM TOMS 15 (1989) 144): its table
is the generator's output (CPU), and on the GPU it is within one ulp of e^x
over the whole normal range, as CUDA's exp is."""

import importlib.util
import io
import os
from contextlib import redirect_stdout

import numpy as np
import pytest

CSRC = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                    "sixtracklib_gb300", "csrc")


def test_table_header_is_the_generators_output():
    spec = importlib.util.spec_from_file_location("gen_exp_table",
                                                  os.path.join(CSRC, "gen_exp_table.py"))
    gen = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(gen)
    buf = io.StringIO()
    with redirect_stdout(buf):
        gen.main()
    with open(os.path.join(CSRC, "exp_table.h")) as f:
        assert f.read() == buf.getvalue()
    hi, lo, l1, l2, inv = gen.table()
    j = np.arange(256)
    # hi + lo is 2^(j/256) to far below an ulp of hi
    assert np.all(np.abs(np.array(hi) - 2.0 ** (j / 256)) <= np.spacing(np.array(hi)))
    assert np.all(np.abs(np.array(lo)) <= 0.5 * np.spacing(np.array(hi)))
    assert (np.float64(l1).view(np.uint64) & np.uint64((1 << 20) - 1)) == 0
    assert abs((l1 + l2) * 256 - np.log(2)) < 1e-16


def ulp_err(got, x):
    """|got - e^x| in ulps of e^x, e^x from numpy (the host libm, correctly
    rounded or within half an ulp plus a little) in extended steps: the
    reference value is exp(x) computed in long double where available."""
    ref = np.exp(x.astype(np.longdouble))
    spacing = np.spacing(ref.astype(np.float64))
    return np.abs(got.astype(np.longdouble) - ref).astype(np.float64) / spacing


@pytest.mark.gpu
def test_within_one_ulp_of_exp():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("GPU tests need a CUDA device")
    from sixtracklib_gb300 import _native

    lib = _native.load()
    rng = np.random.default_rng(17)
    x = np.concatenate([
        rng.uniform(-700, 700, 2_000_000),
        rng.uniform(-1, 1, 1_000_000),
        rng.uniform(-40, 0, 1_000_000),              # the beam fields' range
        -np.logspace(-300, 2.8, 200_000),
        np.logspace(-300, 2.8, 200_000),
        np.array([0.0, -0.0, 5e-324, -5e-324, 699.99, -699.99, 700.0, -700.0, 709.7, -708.4,
                  -745.2, -746.0, 710.0, np.inf, -np.inf, np.nan]),
    ])
    dx = torch.from_numpy(x).cuda()
    dy = torch.empty_like(dx)
    assert lib.st_engine_exp_fast(dx.data_ptr(), dy.data_ptr(), x.size, None) == 0
    torch.cuda.synchronize()
    y = dy.cpu().numpy()
    cuda_exp = torch.exp(dx).cpu().numpy()
    finite = np.isfinite(x) & (np.abs(x) < 700)
    err = ulp_err(y[finite], x[finite])
    err_cuda = ulp_err(cuda_exp[finite], x[finite])
    print(f"exp_fast max {err.max():.3f} ulp, CUDA exp max {err_cuda.max():.3f} ulp, "
          f"differ from CUDA's exp at {(y != cuda_exp).mean():.4f} of the points")
    assert err.max() <= 1.0
    # outside [-700, 700], infinities and NaN: CUDA's exp
    rest = ~finite
    assert np.array_equal(y[rest], cuda_exp[rest], equal_nan=True)
