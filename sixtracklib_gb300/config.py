"""Build and feature settings, as the reference's generated
python/sixtracklib/config.py (config.py.template) lists them.

The reference fixes these when it is compiled; this engine has one build
and takes the map and aperture settings per job or tracker from its
configuration string instead (``track_beambeam4d``, ``track_beambeam6d``,
``track_spacecharge``, ``track_tricub``: "enabled", "skip" or "disabled";
``aperture``: "always", "conditional" or "never"; ``aperture_min_length``,
``x_limit``, ``y_limit``).  The values here are the defaults a job gets
without those keys, which are the reference's default build values
(Settings.cmake.default).
"""

import os

# the engine's shared library, built in the source tree
SHARED_LIB = os.path.join(os.path.dirname(os.path.realpath(__file__)), "lib",
                          "libsixtracklib_gb300.so")

# modules of the build: CUDA only
SIXTRACKLIB_MODULES = {"cuda": True, "opencl": False, "simd": False, "mpfr4": False}

# "enabled" : track the map
# "skip"    : do nothing for elements of this type (success)
# "disabled": tracking through an element of this type fails
TRACK_BEAMBEAM4D = "enabled"
TRACK_BEAMBEAM6D = "enabled"
TRACK_SPACECHARGE = "enabled"
TRACK_TRICUB = "disabled"

# global aperture check after every Drift / DriftExact
APERTURE_CHECK_AT_DRIFT = "always"
APERTURE_CHECK_MIN_DRIFT_LENGTH = 0.0  # [m]
APERTURE_X_LIMIT = 1.0  # [m]
APERTURE_Y_LIMIT = 1.0  # [m]

C99_NAMESPACE_STR = "st_"
C99_NAMESPACE_PREFIX_STR = "st_"
CXX_NAMESPACE_STR = "sixtrack"
CXX_NAMESPACE_PREFIX_STR = "sixtrack::"
