"""GB300-native particle-mesh gravity step for Nyx (sm_103a CUDA behind a C ABI)."""
from .ics import Cosmology, GCONST, InitialConditions, zeldovich_ics  # noqa: F401

__all__ = ["Cosmology", "GCONST", "InitialConditions", "zeldovich_ics", "load_library", "pm"]


def load_library():
    from . import _lib
    return _lib.load()
