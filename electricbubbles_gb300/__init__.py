"""GB300-native implementation of the ElectricBubbles boundary-integral hot path.

The operator applies that GMRES calls every iteration (the Stokes and Laplace layer
potentials of stokesbubb.f / laplace.f, evaluated by the FMMs of cadap*.f / dapif*.f),
the GMRES solves around them and the per-drop spectral routines that feed them, as
CUDA kernels for sm_103a behind the C ABI of include/eb_gb300.h.
"""
from . import configs  # noqa: F401
from ._lib import EbError, library_path, load  # noqa: F401


def Context(*args, **kwargs):  # noqa: N802 - mirrors a class name
    from .api import Context as _C
    return _C(*args, **kwargs)
