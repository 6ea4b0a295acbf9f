"""GB300-native (sm_103a) explicit NOSB peridynamics step.

Drop-in for the mechanics call surface of EricYJA/2D_PD_GPU: C ABI in
include/pd_gb300.h, C++ functions with the reference's names in
include/pd_dropin.h, and this Python mirror (ctypes over the C ABI).

The package directory name starts with a digit, so import it with
``importlib.import_module("2d_pd_gpu_gb300")``.
"""
from . import autotune, native, plates, serve  # noqa: F401
from .native import Batch, Context, PdError, default_params  # noqa: F401
from .plates import make_plate, config_plate_100, config_plate_scale  # noqa: F401

__all__ = ["autotune", "native", "plates", "serve", "Batch", "Context", "PdError", "default_params", "make_plate", "config_plate_100",
           "config_plate_scale"]
