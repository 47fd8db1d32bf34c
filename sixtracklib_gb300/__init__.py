"""GB300-native element-by-element particle tracking (SixTrackLib drop-in)."""

from .cbuffer import CBuffer, CObject
from .beam_elements import *  # noqa: F401,F403
from .beam_elements import Elements
from .particles import (Particles, ParticlesAddr, ParticlesSet,  # noqa: F401
                        calcParticlesDifference, compareParticlesDifference, makeCopy)
# python/sixtracklib/__init__.py: the buffer, track-job and assignment names
# (the library itself is loaded on first use)
from .buffer import AssignAddressItem, Buffer, get_cbuffer_from_obj  # noqa: F401
from .trackjob import CudaTrackJob, TrackJob  # noqa: F401
from .sc_line_density import LineDensityProfileData_create_buffer_assignment  # noqa: F401
from .tricub import TriCub_buffer_create_assign_address_item  # noqa: F401
from . import config  # noqa: F401


def supports(architecture):
    """Whether the engine tracks on `architecture` (config_helper.py:7-8):
    CUDA only."""
    return bool(config.SIXTRACKLIB_MODULES.get(str(architecture).strip().lower(), False))


__version__ = "0.1.0"
