"""GB300-native Barnes-Hut quadrupole gravity step of gravitas (CUDA sm_103a, C-ABI include/gbh.h).

The compute path is libgbh.so only; importing the package does not load it, the first
solver call does, and fails loudly when it has not been built (gravitas_gb300.build.build()).
"""
from . import abi, ics  # noqa: F401

__all__ = ["abi", "ics"]
