"""noa_gb300: GB300-native muon differential cross-sections (NOA PMS DCS).

The compute path is hand-written CUDA for sm_103a behind the C ABI of
include/noa_dcs.h (noa_gb300/libnoa_dcs.so); this package is the host-side
mirror of the reference's noa::pms::dcs::cuda surface.  Build the native
library with `python -m noa_gb300.build`.
"""
from .elements import (ELEMENTS, ELECTRON_MASS, MUON_MASS, STANDARD_ROCK, TAU_MASS, X_FRACTION,
                       AtomicElement)
from . import dcs

__all__ = ["dcs", "AtomicElement", "STANDARD_ROCK", "MUON_MASS", "TAU_MASS", "ELECTRON_MASS",
           "X_FRACTION", "ELEMENTS"]
