"""bgk2d_gpu_gb300 -- GB300 (sm_103a) D2Q9 BGK time step of BGK2D behind a C ABI.

`Solver` mirrors the reference's per-step interface (boundaries / propagation / collision and
the diagnostic readers) over libbgk2d_gb300.so; there is no CPU execution path.
"""
from ._lib import BgkError, load, lib_path  # noqa: F401
from .solver import Batch, Server, Solver, read_namelist, CX, CY, WEIGHTS  # noqa: F401

__all__ = ["Batch", "Server", "Solver", "BgkError", "load", "lib_path", "read_namelist", "CX", "CY", "WEIGHTS"]
