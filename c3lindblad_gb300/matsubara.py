"""Impurity Green function on a fermionic Matsubara grid from the device response.

Counterparts of the reference's explicit ``MatsubaraGrid`` / ``matsubara_grid``
(``src/c3l/matsubara/grid.py:17-98, 169-212``) and ``component_matsubara_green``
(``src/c3l/matsubara/solver.py:16-68``).  The response is
``component_retarded_matrix_green_shifts`` at the grid's distinct upper
half-plane points z = i|omega_n| (one Arnoldi basis per source and channel on
the device, all points from it); negative frequencies receive
G(-i omega) = G(i omega)^dagger.  ``component_matsubara_green`` also accepts the
reference's own grid objects (anything with ``upper_shifts`` and
``from_upper``), DLR grids included.  The self-energy and Dyson steps of
``solve_matsubara`` need the physical model (setup) and are not part of this
package.
"""

from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from .response import component_retarded_matrix_green_shifts

_MATSUBARA_TOLERANCE = 1.0e-8


@dataclass(frozen=True, eq=False)
class MatsubaraGrid:
    """Fermionic points i omega_n, omega_n = (2n + 1) pi / beta, in the caller's index order."""

    beta: float
    indices: np.ndarray
    kind: str = "explicit"
    _upper_odd: np.ndarray = field(init=False, repr=False)
    _upper_index: np.ndarray = field(init=False, repr=False)

    def __post_init__(self) -> None:
        beta = float(self.beta)
        if not np.isfinite(beta) or beta <= 0.0:
            raise ValueError("beta must be finite and positive")
        raw = np.asarray(self.indices)
        if raw.ndim != 1 or raw.size == 0 or not np.issubdtype(raw.dtype, np.integer):
            raise ValueError("indices must be a nonempty integer vector")
        indices = raw.astype(np.int64)
        if np.unique(indices).size != indices.size:
            raise ValueError("Matsubara indices must be unique")
        if self.kind != "explicit":
            raise ValueError("only explicit grids are built here (DLR grids need pydlr)")
        indices.setflags(write=False)
        odd, inverse = np.unique(np.abs(2 * indices + 1), return_inverse=True)
        object.__setattr__(self, "beta", beta)
        object.__setattr__(self, "indices", indices)
        object.__setattr__(self, "_upper_odd", odd)
        object.__setattr__(self, "_upper_index", inverse.astype(np.int64).reshape(-1))

    def __len__(self) -> int:
        return int(self.indices.size)

    @property
    def omega_n(self) -> np.ndarray:
        return (2 * self.indices + 1) * np.pi / self.beta

    @property
    def iw(self) -> np.ndarray:
        return 1j * self.omega_n

    @property
    def upper_shifts(self) -> np.ndarray:
        """Distinct points i|omega_n|, increasing."""
        return 1j * self._upper_odd * np.pi / self.beta

    def from_upper(self, values) -> np.ndarray:
        """Values at ``upper_shifts`` ([k] or [k, m, m]) onto the grid; negative
        frequencies take the conjugate (transpose)."""
        upper = np.asarray(values, dtype=np.complex128)
        if upper.ndim not in (1, 3) or upper.shape[0] != self._upper_odd.size:
            raise ValueError("values must have shape (len(upper_shifts),) or (len(upper_shifts), m, m)")
        if upper.ndim == 3 and upper.shape[1] != upper.shape[2]:
            raise ValueError("matrix values must be square")
        out = upper[self._upper_index].copy()
        negative = self.indices < 0
        if upper.ndim == 1:
            out[negative] = out[negative].conj()
        else:
            out[negative] = out[negative].conj().swapaxes(1, 2)
        return out


def matsubara_grid(beta: float, *, indices=None, omega_n=None, n_iw: int | None = None) -> MatsubaraGrid:
    """An explicit grid from exactly one of ``indices``, ``omega_n`` (real, or
    purely imaginary points) or ``n_iw`` (n = -n_iw .. n_iw - 1); frequencies
    must lie on this beta's fermionic lattice to relative accuracy 1e-8."""
    given = [v is not None for v in (indices, omega_n, n_iw)]
    if sum(given) != 1:
        raise ValueError("give exactly one of indices, omega_n, or n_iw")
    b = float(beta)
    if not np.isfinite(b) or b <= 0.0:
        raise ValueError("beta must be finite and positive")
    if n_iw is not None:
        if isinstance(n_iw, bool) or not isinstance(n_iw, (int, np.integer)) or n_iw <= 0:
            raise ValueError("n_iw must be a positive integer")
        return MatsubaraGrid(b, np.arange(-int(n_iw), int(n_iw)))
    if indices is not None:
        return MatsubaraGrid(b, np.asarray(indices))
    w = np.asarray(omega_n)
    if np.iscomplexobj(w):
        if np.any(np.abs(w.real) > _MATSUBARA_TOLERANCE * np.maximum(np.abs(w), 1.0)):
            raise ValueError("complex Matsubara points must be purely imaginary")
        w = w.imag
    w = np.asarray(w, dtype=np.float64)
    if w.ndim != 1 or w.size == 0 or not np.all(np.isfinite(w)):
        raise ValueError("omega_n must be a finite nonempty vector")
    odd = w * b / np.pi
    nearest = np.rint(odd)
    if (np.any(np.abs(odd - nearest) > _MATSUBARA_TOLERANCE * np.maximum(np.abs(odd), 1.0))
            or np.any(nearest.astype(np.int64) % 2 == 0)):
        raise ValueError("omega_n are not fermionic Matsubara frequencies for this beta")
    return MatsubaraGrid(b, (nearest.astype(np.int64) - 1) // 2)


@dataclass(frozen=True, eq=False)
class MatsubaraGreen:
    """Impurity G(i omega_n) from one response operator (axes n, sink, source)."""

    grid: object
    sites: tuple
    green: np.ndarray
    upper: object

    @property
    def max_relative_residual(self) -> float:
        """Largest Arnoldi relative residual over sources, channels and shifts."""
        return float(max(np.max(self.upper.addition_relative_residuals),
                         np.max(self.upper.removal_relative_residuals)))


def component_matsubara_green(operator, sources, grid, *, maximum_krylov_dimension: int = 320,
                              residual_tolerance: float = 1.0e-10, minimum_krylov_dimension: int = 16,
                              check_interval: int = 8) -> MatsubaraGreen:
    """G(i omega_n) for the impurity sources: one device Arnoldi basis per source
    and channel shared by all points i|omega_n| (``solver.py:37-68``)."""
    if not (hasattr(grid, "upper_shifts") and hasattr(grid, "from_upper")):
        raise TypeError("grid must be a MatsubaraGrid")
    upper = component_retarded_matrix_green_shifts(
        operator, sources, np.asarray(grid.upper_shifts, dtype=np.complex128),
        maximum_krylov_dimension=maximum_krylov_dimension, residual_tolerance=residual_tolerance,
        minimum_krylov_dimension=minimum_krylov_dimension, check_interval=check_interval)
    return MatsubaraGreen(grid=grid, sites=upper.sites, green=grid.from_upper(upper.retarded), upper=upper)
