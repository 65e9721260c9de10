"""GB300-native FX correlator engine: drop-in for the reference's libcorr_cuda.so.

The product is the C-ABI shared library built from csrc/ (include/corr_cuda.h,
include/corr_gb300.h, include/corr_writer.h). This package builds it (build.py),
binds it with ctypes (abi.py), and mirrors the reference's host-side wrapper
(correlator.py) and the device-resident engine (engine.py). frontend.py drives
the on-device synthetic front end, writer.py the output file sets, phase.py fits
delays from rows; synth.py generates the seeded workloads.
"""

from . import abi
from .abi import CorrError
from .correlator import Correlator, make_config, plan_query, set_device_map
from .engine import FxEngine

__all__ = ["abi", "CorrError", "Correlator", "make_config", "plan_query", "set_device_map",
           "FxEngine"]
