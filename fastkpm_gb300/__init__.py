"""fastkpm_gb300 -- GB300-native stochastic Chebyshev (KPM) engine.

Python mirror of FastKPM's fkpm interface over the C ABI of
libfastkpm_gb300.so (hand-written sm_103a kernels). See include/fastkpm.h for
the drop-in C++ interface and include/fastkpm_gb300.h for the C ABI.
"""
from . import _lib
from .engine import (Batch, Engine, EnergyScale, RNG, SpMatBsr, device_count, expansion_coefficients, jackson_kernel,
                     mk_engine, moment_product, probe_correlated, probe_identity, probe_uncorrelated)

__all__ = ["Batch", "Engine", "EnergyScale", "RNG", "SpMatBsr", "device_count", "expansion_coefficients", "jackson_kernel",
           "mk_engine", "moment_product", "probe_correlated", "probe_identity", "probe_uncorrelated"]


def library():
    """The loaded libfastkpm_gb300.so (raises if it is not built)."""
    return _lib.load()
