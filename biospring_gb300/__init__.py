"""biospring_gb300 -- BioSpring's per-step force-and-integrate loop on one GB300 (sm_103a).

The CUDA kernels and their C ABI (``include/biospring_gb300.h``) live in
``libbiospring_gb300.so``; :class:`SpringNetwork` mirrors the reference engine's interface
over that ABI. There is no CPU fallback: if the library is missing, import of the network
raises when it is first used.
"""

from .capi import BsConfig, BsError, default_config, parse_msp  # noqa: F401
from .network import SpringNetwork  # noqa: F401

__all__ = ["SpringNetwork", "BsConfig", "BsError", "default_config", "parse_msp"]
