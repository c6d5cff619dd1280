"""fastpli_gb300 — GB300 (sm_103a) forward model of 3D polarized light imaging.

A drop-in for the compiled back ends of fastpli's ``Simpli``: the voxelizer
(``_Generator``) and the ray march (``_Simulator``), both hand-written CUDA
behind the C ABI in ``include/fastpli_gb300.h``.  ``Simpli`` mirrors the
reference's user API for the forward model.  There is no CPU fallback: the
native library must load or every call raises.
"""

from . import synth  # noqa: F401
from .simpli import Simpli  # noqa: F401
from .simulation import _Generator, _Simulator  # noqa: F401

__version__ = "0.1.0"


def native_library():
    """Load (building if needed) and return the ctypes handle."""
    from . import _native
    return _native.load()
