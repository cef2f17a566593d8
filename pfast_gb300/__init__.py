"""pfast_gb300 -- GB300 (sm_103a) implementation of PFAST's traveltime-and-gradient
hot path: fast-sweeping Eikonal solves, Huygens reflection traveltimes and
adjoint-state gradients, behind a C ABI (include/pfast_gb300.h).

The CUDA library is the only compute path.  Importing this package loads it
and raises if it was not built.
"""
from ._capi import lib as _lib

_lib()  # fail loudly when the CUDA library is missing

from .api import *  # noqa: E402,F401,F403
from . import api, synth, io, workloads  # noqa: E402,F401

__version__ = "0.1.0"
