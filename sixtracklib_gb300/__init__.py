"""GB300-native element-by-element particle tracking (SixTrackLib drop-in)."""

from .cbuffer import CBuffer, CObject
from .beam_elements import *  # noqa: F401,F403
from .beam_elements import Elements
from .particles import (Particles, ParticlesSet, calcParticlesDifference,  # noqa: F401
                        compareParticlesDifference, makeCopy)

__version__ = "0.1.0"
