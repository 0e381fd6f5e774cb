"""tdscha_gb300: GB300-native (sm_103a) TD-SCHA Lanczos linear-response engine.

Drop-in for the reference's `tdscha.DynamicalLanczos.Lanczos` hot path: the
ensemble-averaged D3/D4 anharmonic operator applied to Lanczos vectors runs as
CUDA kernels behind a C ABI (include/tdscha_gb300.h); the Python layer mirrors
the reference's API.
"""
from . import _native  # noqa: F401
from .DynamicalLanczos import Lanczos, MODE_GB300  # noqa: F401

__all__ = ["Lanczos", "MODE_GB300"]
