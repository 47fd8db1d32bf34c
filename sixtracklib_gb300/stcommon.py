"""Names of the reference's ``sixtracklib.stcommon`` module that user code
imports for this path (python/sixtracklib/stcommon.py).

* The q-Gaussian helpers of ``internal/math_qgauss.h:100-190`` (used to set
  up SCQGaussProfile kicks): ``Math_q_gauss_cq``,
  ``Math_sqrt_beta_from_gauss_sigma``, ``Math_q_gauss_exp_q``,
  ``Math_q_gauss`` (optionally shifted by ``mu``) and the support limits,
  computed here in Python with the reference's formulas.
* The architecture buffer ids and status values as ctypes values (``.value``
  gives the number), and null handles (``st_NullBuffer``: None, which is
  what a failed C call returns through ctypes here).
* Every ``st_*`` function of the engine's C ABI that the package binds with
  a signature (:mod:`sixtracklib_gb300._native`), resolved on first use.
"""

from __future__ import annotations

import ctypes as ct
from math import sqrt

import numpy as np

from . import buffer as _buffer
from .beam_elements import q_gauss_cq as _q_gauss_cq
from .trackjob import st_ParticlesAddr  # noqa: F401  (stcommon.py:517-542)

SIXTRL_MATH_QGAUSSIAN_Q_EPS = 1e-6

st_ARCH_STATUS_SUCCESS = ct.c_int32(0)
st_ARCH_STATUS_GENERAL_FAILURE = ct.c_int32(-1)
st_TRACK_SUCCESS = ct.c_int32(0)
st_ARCH_ILLEGAL_BUFFER_ID = ct.c_uint64(_buffer.ARCH_ILLEGAL_BUFFER_ID)
st_ARCH_PARTICLES_BUFFER_ID = ct.c_uint64(_buffer.ARCH_PARTICLES_BUFFER_ID)
st_ARCH_BEAM_ELEMENTS_BUFFER_ID = ct.c_uint64(_buffer.ARCH_BEAM_ELEMENTS_BUFFER_ID)
st_ARCH_OUTPUT_BUFFER_ID = ct.c_uint64(_buffer.ARCH_OUTPUT_BUFFER_ID)
st_ARCH_ELEM_BY_ELEM_CONFIG_BUFFER_ID = ct.c_uint64(_buffer.ARCH_ELEM_BY_ELEM_CONFIG_BUFFER_ID)
st_ARCH_PARTICLE_ADDR_BUFFER_ID = ct.c_uint64(_buffer.ARCH_PARTICLE_ADDR_BUFFER_ID)
st_ARCH_MIN_USER_DEFINED_BUFFER_ID = ct.c_uint64(_buffer.ARCH_MIN_USER_DEFINED_BUFFER_ID)
st_ARCH_EXTERNAL_BUFFER_ID = ct.c_uint64(_buffer.ARCH_EXTERNAL_BUFFER_ID)
st_ARCH_MAX_USER_DEFINED_BUFFER_ID = ct.c_uint64(_buffer.ARCH_MAX_USER_DEFINED_BUFFER_ID)

st_NullBuffer = None
st_NullParticles = None
st_NullTrackJob = None
st_NullAssignAddressItem = None


# -------------------------------------------------- q-Gaussian (math_qgauss.h)
def Math_q_gauss_cq(q):
    """Normalisation c_q of the q-Gaussian (q < 3)."""
    assert q < 3.0
    return _q_gauss_cq(q)


def Math_sqrt_beta_from_gauss_sigma(sigma):
    """sqrt(beta) of the Gaussian (q = 1) of rms ``sigma``: 1 / (sqrt(2) sigma)."""
    assert sigma > 0
    return 1.0 / (sqrt(2.0) * sigma)


def Math_q_gauss_exp_q(x, q):
    """The q-exponential [1 + (1 - q) x]_+^(1 / (1 - q)), exp(x) for q = 1."""
    assert q < 3.0
    one_minus_q = 1.0 - q
    if abs(one_minus_q) >= SIXTRL_MATH_QGAUSSIAN_Q_EPS:
        u = max(1.0 + one_minus_q * x, 0.0)
        return u ** (1.0 / one_minus_q)
    return float(np.exp(x))


def Math_q_gauss(x, q, sqrt_beta, mu=None):
    """The normalised q-Gaussian at ``x`` (centred at ``mu`` if given)."""
    assert q < 3.0 and sqrt_beta > 0.0
    if mu is not None:
        x = x - mu
    cq = Math_q_gauss_cq(q)
    return (sqrt_beta / cq) * Math_q_gauss_exp_q(-(sqrt_beta * sqrt_beta * x * x), q)


def Math_q_gauss_min_support(q, sqrt_beta):
    """Lower end of the support: -1 / sqrt(beta (1 - q)) for q < 1, else -1e10."""
    assert q < 3.0 and sqrt_beta > 0.0
    return -1e10 if q >= 1.0 else -1.0 / sqrt(sqrt_beta * sqrt_beta * (1.0 - q))


def Math_q_gauss_max_support(q, sqrt_beta):
    """Upper end of the support: 1 / sqrt(beta (1 - q)) for q < 1, else 1e10."""
    assert q < 3.0 and sqrt_beta > 0.0
    return 1e10 if q >= 1.0 else 1.0 / sqrt(sqrt_beta * sqrt_beta * (1.0 - q))


# ------------------------------------------------------------ C functions
def __getattr__(name):
    if name.startswith("st_"):
        from . import _native

        if name in _native._SIGNATURES:
            return getattr(_native.load(), name)
        raise AttributeError(f"{name} is not part of this engine's bound C ABI "
                             f"(see include/sixtracklib_gb300.h and _native)")
    raise AttributeError(name)
