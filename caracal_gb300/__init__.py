"""GB300-native RPMD engine for Caracal's dynamic / calc_rate hot path.

The compute path is the CUDA library built from ``csrc/`` (sm_103a); this
package only loads it (``_lib``) and mirrors its C-ABI in Python
(``engine``).  There is no CPU fallback.
"""
from . import units  # noqa: F401
from ._lib import CaracalError, lib  # noqa: F401
from .engine import EVBPair, QMDFFForceField, RPMDBatch, RPMDEngine, WaterBox, egrad_brh2, egrad_ch4h, egrad_ch4oh, egrad_geh4oh, egrad_h3, egrad_oh3  # noqa: F401

__all__ = ["RPMDEngine", "RPMDBatch", "QMDFFForceField", "EVBPair", "WaterBox", "egrad_h3", "egrad_ch4h", "egrad_ch4oh", "egrad_geh4oh", "egrad_brh2", "egrad_oh3", "CaracalError", "lib",
           "units"]
