"""pfast_gb300 -- GB300 (sm_103a) implementation of PFAST's traveltime-and-gradient
hot path: fast-sweeping Eikonal solves, Huygens reflection traveltimes and
adjoint-state gradients, behind a C ABI (include/pfast_gb300.h).

The CUDA library is the only compute path.  It is loaded by the first call into
it (creating a Context, or any reference-signature function), which raises if it
was not built; there is no CPU fallback.  The seeded workload generators
(`synth`, `workloads.c3_inputs`) are plain numpy and do not load it.
"""
from .api import *  # noqa: F401,F403
from . import api, synth, io, workloads  # noqa: F401


def load_library():
    """Load libpfast_gb300.so now (raises ImportError if it was not built)."""
    from ._capi import lib
    return lib()


__version__ = "0.1.0"
