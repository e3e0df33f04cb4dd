"""lbswim for GB300: the gpu-swimmers coupled step on hand-written sm_103a kernels.

Modules mirror the reference package: ``lb`` (Lattice), ``swimmers``
(CommonParams, Array), ``tracers`` (Array), ``shared`` and ``System``.
"""
from . import _lib  # noqa: F401  (fails loudly if the library is missing)
