"""GB300 preconditioned Krylov library: drop-in for MTJ's sparse iterative path.

``mtjg.sparse`` mirrors ``no.uib.cipr.matrix.sparse`` over the C ABI of
``include/mtjg.h`` (libmtjg.so, hand-written sm_103a CUDA).
``mtjg.workloads`` builds the seeded synthetic systems.
"""
from . import _lib  # noqa: F401
from ._lib import load  # noqa: F401

__all__ = ["sparse", "workloads", "load"]
