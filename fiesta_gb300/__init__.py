"""fiesta_gb300 — GB300 (sm_103a) implementation of FIESTA's per-RK-stage
right-hand side and update (cart2d / cart3d modules), behind a C ABI
(include/fst.h, fiesta_gb300/libfst.so)."""
from . import abi  # noqa: F401
from .solver import (Cart2D, Cart3D, FstError, Solver, initial_conditions,  # noqa: F401
                     lib, rkAdvance)
