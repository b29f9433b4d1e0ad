"""opencamlib_gb300 -- GB300-native drop-cutter and push-cutter.

Python mirror of the reference library's operation API (opencamlib's `ocl`
module: STLSurf, the milling cutters, BatchDropCutter, PathDropCutter,
AdaptivePathDropCutter, BatchPushCutter, ...) over the C ABI of
libocl_gb300.so.  All computation runs in the CUDA library; there is no CPU
fallback.
"""
from ._native import DeviceMesh, DropBatch, OclError, Server, device_available, lib  # noqa: F401
from .cutters import (BallConeCutter, BallCutter, BullConeCutter, BullCutter, CompBallCutter, CompCylCutter,  # noqa: F401
                      CompositeCutter, ConeConeCutter, ConeCutter, CylConeCutter, CylCutter, MillingCutter)
from .api import *  # noqa: F401,F403
