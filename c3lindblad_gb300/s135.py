"""The full S1 + S3 + S5 response action (the rank-five shell) on the device.

Counterparts of the reference's ``CompiledFullS135Action`` and
``FullS135ResponseOperator`` (``src/c3l/cc/s135_full.py:101-361``).  The
reference enumerates BCH response plans with a rank-five input placeholder
and projects them tile by tile; here the same action is the EOM sigma program
compiled for response vectors of degrees 1, 3 and 5 (``EOMPlan(...,
space="S135")``: the symbolic expansion keeps output degrees {1, 3, 5}), so
its contractions, rest forms, pair GEMMs and epilogue run on the same kernels
as the S13 sigma.  The vector layout is the reference's: the S13 coordinates,
then the rank-five shell block by block (``layout.eom_coordinates``).  The
operator is a ``ComponentSigmaOperator``, so every response driver accepts it;
the S13 sources are padded with zeros to its dimension.
"""

from __future__ import annotations

import time

import numpy as np

from .response import ComponentEOMContext, ComponentEOMProblem, ComponentSigmaOperator


class CompiledFullS135Action:
    """The S135 action at the amplitudes of an S13 ``ComponentEOMContext``
    (same static problem, response spin, charge and interaction scale)."""

    def __init__(self, context: ComponentEOMContext, *, materialization_batch_size: int = 16):
        if materialization_batch_size <= 0 or materialization_batch_size > 16:
            raise ValueError("materialization_batch_size must be in [1,16]")
        started = time.perf_counter()
        p = context.problem
        self.context = context
        self.problem = ComponentEOMProblem(p.static, p.response_spin, p.charge, space="S135")
        self.full_context = ComponentEOMContext(self.problem, context.amplitudes,
                                                interaction_scale=getattr(context, "interaction_scale", 1.0))
        self.p_dimension = int(p.plan.dimension)
        self.dimension = int(self.problem.plan.dimension)
        self.s5_dimension = self.dimension - self.p_dimension
        self.compile_seconds = time.perf_counter() - started


class FullS135ResponseOperator(ComponentSigmaOperator):
    """Exact right action on the complete S1 + S3 + S5 space (device)."""

    def __init__(self, action: CompiledFullS135Action, *, s5_tile_size: int = 16384):
        if s5_tile_size <= 0:
            raise ValueError("s5_tile_size must be positive")
        super().__init__(action.full_context)
        self.action = action
        self.p_dimension = action.p_dimension
        self.s5_dimension = action.s5_dimension
        self.s5_tile_size = int(s5_tile_size)  # the device action needs no tiling; kept for the signature

    def matvec(self, vector) -> np.ndarray:
        arr = np.asarray(vector, dtype=np.complex128)
        if arr.shape != (self.dimension,) or not np.all(np.isfinite(arr)):
            raise ValueError("the full-S135 input has the wrong shape or is nonfinite")
        return super().matvec(arr)


def rapidity_diagonal(operator: FullS135ResponseOperator) -> np.ndarray:
    """The quadratic response diagonal on the S135 coordinates (the sum of the
    rapidities of each coordinate's modes; ``s135_full.py:273-293``)."""
    return operator.context.problem.plan.diagonal.copy()


__all__ = ["CompiledFullS135Action", "FullS135ResponseOperator", "rapidity_diagonal"]
