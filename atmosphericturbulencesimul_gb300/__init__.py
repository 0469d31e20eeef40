"""GB300-native engine for the wavefront-series hot path of AtmosphericTurbulenceSimul.

The compute path is libatmwfs.so (hand-written CUDA for sm_103a behind the C
ABI in include/atmwfs.h); this package is its Python front end.
"""
from .engine import (MODE_PHASE, MODE_REF, MODE_SCI, InstanceSpec, Series, fft2d, fresnel,  # noqa: F401
                     layer_planes, master_screen)

__version__ = "0.1.0"
