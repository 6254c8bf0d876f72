"""GB300-native block-structured AMR hot path (Parthenon-compatible semantics).

Native library: libparthenon_gb300.so (C ABI in include/parthenon_gb300.h), built with
`parthenon_gb300.build.build()`. This package is the host-side mirror of the
reference's mesh / exchange / driver interface; all compute runs in the library.
"""
from .mesh import Mesh  # noqa: F401
from .driver import RK2Driver, StageConfig  # noqa: F401
from .gmg import CompositeMultigrid, GmgSolver  # noqa: F401
from .amr import AMRDriver, RefinementCriterion, SparseMinMaxCriterion  # noqa: F401
from . import history, problems  # noqa: F401
from ._native import NativeError  # noqa: F401

__all__ = ["Mesh", "RK2Driver", "StageConfig", "GmgSolver", "CompositeMultigrid", "AMRDriver", "RefinementCriterion",
           "SparseMinMaxCriterion", "history", "problems", "NativeError"]
