"""nesf -- GB300-native interface-flux step for NumericalEarth.jl.

Host-side mirror of the reference's flux interface: parameter types with the
reference names and defaults (`params`), field bundles (`fields`), seeded
synthetic workloads (`synthetic`) and the entry points of the C ABI
(`api`, `_lib`). Compute runs only in libnesf.so (CUDA, sm_103a).
"""
from . import _abi, params, fields, synthetic  # noqa: F401
from .params import *  # noqa: F401,F403

__version__ = "0.1.0"
