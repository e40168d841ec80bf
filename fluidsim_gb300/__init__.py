"""fluidsim_gb300 — GB300-native (sm_103a) FluidSim particle hot path.

The product is the native library ``_build/libfluidsim.so`` behind the C ABI
``include/fluidsim.h``; this package holds its sources (``csrc/``), the build
recipe (``build.py``), a ctypes binding (``api.py``) and the benchmark cases
(``cases.py``).
"""
from . import api, cases  # noqa: F401
from .api import Simulation, load  # noqa: F401
