"""Impurity Green function on a fermionic Matsubara grid from the device response.

Counterparts of the reference's explicit ``MatsubaraGrid`` / ``matsubara_grid``
(``src/c3l/matsubara/grid.py:17-98, 169-212``) and ``component_matsubara_green``
(``src/c3l/matsubara/solver.py:16-68``).  The response is
``component_retarded_matrix_green_shifts`` at the grid's distinct upper
half-plane points z = i|omega_n| (one Arnoldi basis per source and channel on
the device, all points from it); negative frequencies receive
G(-i omega) = G(i omega)^dagger.  ``component_matsubara_green`` also accepts the
reference's own grid objects (anything with ``upper_shifts`` and
``from_upper``), DLR grids included.

``solve_matsubara`` chains the device static solve, EOM context, sources and
Matsubara response with the self-energy Sigma = G0^-1 - G^-1 and the Dyson
equation on the host (``src/c3l/matsubara/solver.py:100-232``,
``src/c3l/matsubara/dyson.py:15-175``,
``src/c3l/spectra/reconstruction.py:174-257``): small dense solves of the
impurity block per grid point, read from the physical one-body model that a
``ProblemSpec`` carries (E, gamma_loss, gamma_gain, interaction sites) or from
the reference's own ``FermionicLindbladModel``.
"""

from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from .response import component_retarded_matrix_green_shifts
from .spectra import matrix_auxiliary_self_energy

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


# ------------------------------------------------------ self-energy and Dyson
@dataclass(frozen=True)
class PhysicalModel:
    """The one-body Lindblad model of one spin block (the attributes of the
    reference's ``FermionicLindbladModel`` that the Dyson steps read)."""

    E: np.ndarray
    gamma_loss: np.ndarray
    gamma_gain: np.ndarray
    interaction_sites: tuple
    has_interactions: bool
    impurity_site: int = 0

    @property
    def n_sites(self) -> int:
        return int(self.E.shape[0])


def physical_model(obj) -> PhysicalModel:
    """The physical model of a ``ProblemSpec``, a compiled problem carrying one,
    or a reference model (duck-typed: ``E``, ``gamma_loss``, ``gamma_gain``,
    ``interaction_sites``, ``has_interactions``)."""
    if isinstance(obj, PhysicalModel):
        return obj
    spec = getattr(obj, "spec", obj)
    if hasattr(spec, "has_model"):
        if not spec.has_model:
            raise ValueError("the problem spec carries no physical model (E, gamma_loss, gamma_gain)")
        return PhysicalModel(np.asarray(spec.model_E, np.complex128), np.asarray(spec.model_gamma_loss, np.complex128),
                             np.asarray(spec.model_gamma_gain, np.complex128),
                             tuple(int(v) for v in spec.interaction_sites), bool(spec.has_interactions),
                             int(spec.impurity_site))
    if all(hasattr(obj, a) for a in ("E", "gamma_loss", "gamma_gain", "interaction_sites", "has_interactions")):
        return PhysicalModel(np.asarray(obj.E, np.complex128), np.asarray(obj.gamma_loss, np.complex128),
                             np.asarray(obj.gamma_gain, np.complex128), tuple(int(v) for v in obj.interaction_sites),
                             bool(obj.has_interactions), int(getattr(obj, "impurity_site", 0)))
    raise TypeError("model must be a ProblemSpec with a physical model or a FermionicLindbladModel")


def impurity_sites(model, sites=None) -> tuple:
    """The impurity block S (``dyson.py:15-40``): default the interaction sites;
    every interacting site must be included, or G0^-1 - G^-1 is not the
    impurity self-energy."""
    m = physical_model(model)
    chosen = tuple(m.interaction_sites if sites is None else sites)
    if not chosen:
        raise ValueError("at least one impurity site is required")
    if any(isinstance(v, (bool, np.bool_)) or not isinstance(v, (int, np.integer)) for v in chosen):
        raise TypeError("impurity sites must be integers")
    chosen = tuple(int(v) for v in chosen)
    if any(not 0 <= v < m.n_sites for v in chosen):
        raise ValueError("an impurity site is outside the model")
    if len(set(chosen)) != len(chosen):
        raise ValueError("impurity sites must be unique")
    if m.has_interactions and not set(m.interaction_sites) <= set(chosen):
        raise ValueError("impurity sites must include every interaction site")
    return chosen


def noninteracting_retarded_green(model, shifts, sites=None) -> np.ndarray:
    """[(z - E + i(gamma_loss + gamma_gain))^-1]_SS at each shift z (``dyson.py:43-64``)."""
    m = physical_model(model)
    block = list(impurity_sites(m, sites))
    z = np.asarray(shifts, dtype=np.complex128)
    if z.ndim != 1 or z.size == 0 or not np.all(np.isfinite(z)):
        raise ValueError("shifts must be a finite nonempty vector")
    n = m.n_sites
    eye = np.eye(n, dtype=np.complex128)
    effective = m.E - 1j * (m.gamma_loss + m.gamma_gain)
    lhs = z[:, None, None] * eye[None] - effective[None]
    cols = np.broadcast_to(eye[:, block], (z.size, n, len(block)))
    return np.ascontiguousarray(np.linalg.solve(lhs, cols)[:, block, :])


def matsubara_noninteracting_green(model, grid, sites=None) -> np.ndarray:
    """The noninteracting impurity block on a Matsubara grid (``dyson.py:67-74``)."""
    return grid.from_upper(noninteracting_retarded_green(model, grid.upper_shifts, sites))


@dataclass(frozen=True, eq=False)
class MatsubaraSelfEnergy:
    """Auxiliary Dyson quantities on a Matsubara grid (axes n, a, b); the
    hybridization is Delta = i omega_n - h - G0^-1 with h = E_SS."""

    grid: object
    sites: tuple
    one_body: np.ndarray
    noninteracting: np.ndarray
    hybridization: np.ndarray
    self_energy: np.ndarray
    G0_condition_number: np.ndarray
    G_condition_number: np.ndarray
    conditioning_limited: np.ndarray


def matsubara_self_energy(model, grid, green, *, sites=None, conditioning_limit: float = 1.0e10
                          ) -> MatsubaraSelfEnergy:
    """Sigma = G0^-1 - G^-1 for ``green`` on ``grid`` (``dyson.py:98-133``)."""
    m = physical_model(model)
    block = impurity_sites(m, sites)
    G = np.asarray(green, dtype=np.complex128)
    if G.shape != (len(grid), len(block), len(block)) or not np.all(np.isfinite(G)):
        raise ValueError("green must be finite with shape (len(grid), len(sites), len(sites))")
    G0 = matsubara_noninteracting_green(m, grid, block)
    result = matrix_auxiliary_self_energy(G0, G, conditioning_limit=conditioning_limit)
    h = m.E[np.ix_(block, block)].copy()
    eye = np.eye(len(block), dtype=np.complex128)
    hyb = grid.iw[:, None, None] * eye[None] - h[None] - np.linalg.inv(G0)
    return MatsubaraSelfEnergy(grid=grid, sites=block, one_body=h, noninteracting=G0, hybridization=hyb,
                               self_energy=result.retarded, G0_condition_number=result.G0_condition_number,
                               G_condition_number=result.G_condition_number,
                               conditioning_limited=result.conditioning_limited)


def matsubara_dyson_green(grid, one_body, hybridization, self_energy) -> np.ndarray:
    """G = [i omega_n - h - Delta(i omega_n) - Sigma(i omega_n)]^-1 (``dyson.py:136-164``)."""
    delta = np.asarray(hybridization, dtype=np.complex128)
    sigma = np.asarray(self_energy, dtype=np.complex128)
    h = np.asarray(one_body, dtype=np.complex128)
    if (delta.ndim != 3 or delta.shape[0] != len(grid) or delta.shape[1] != delta.shape[2]
            or sigma.shape != delta.shape or h.shape != delta.shape[1:]):
        raise ValueError("one_body, hybridization, and self_energy have incompatible shapes")
    if not all(np.all(np.isfinite(v)) for v in (delta, sigma, h)):
        raise ValueError("Dyson inputs must be finite")
    eye = np.eye(h.shape[0], dtype=np.complex128)
    lhs = grid.iw[:, None, None] * eye[None] - h[None] - delta - sigma
    return np.linalg.solve(lhs, np.broadcast_to(eye, lhs.shape))


@dataclass(frozen=True, eq=False)
class MatsubaraImpuritySolution:
    """CCSD + EOM impurity solution on a Matsubara grid: ``green`` and
    ``self_energy`` have axes (n, a, b) over ``sites``; :meth:`dyson` inserts
    the self-energy into another hybridization."""

    grid: object
    sites: tuple
    rank: str
    response_spin: int
    green: np.ndarray
    self_energy: np.ndarray
    noninteracting: np.ndarray
    hybridization: np.ndarray
    one_body: np.ndarray
    amplitudes: np.ndarray
    static_residual: float | None
    response: MatsubaraGreen
    dyson_terms: MatsubaraSelfEnergy

    def dyson(self, hybridization) -> np.ndarray:
        """[i omega_n - h - Delta - Sigma]^-1 for a target ``hybridization``."""
        return matsubara_dyson_green(self.grid, self.one_body, hybridization, self.self_energy)


def solve_matsubara(model, grid, *, sites=None, rank: str = "S13", response_spin: int = 0, amplitudes=None,
                    policy=None, precision: str = "mixed", maximum_krylov_dimension: int = 320,
                    residual_tolerance: float = 1.0e-10, minimum_krylov_dimension: int = 16,
                    check_interval: int = 8) -> MatsubaraImpuritySolution:
    """Solve CCSD and the EOM response on the device, returning G(i omega_n) and
    Sigma(i omega_n) (``src/c3l/matsubara/solver.py:100-232``).

    ``model`` is a ``ComponentStaticProblem`` or ``ProblemSpec`` carrying the
    physical model, or the reference's ``ComponentStaticProblem`` /
    ``FactorizedCCProblem``.  Converged ``amplitudes`` skip the static solve.
    The reference's ``platform``/``production`` switches select its NumPy or
    JAX backends and have no counterpart here: the device path always runs
    (``precision`` picks the static solve's form).  ``rank="S135"`` responds
    through ``FullS135ResponseOperator`` (the rank-five shell).
    """
    from .response import (ComponentEOMProblem, ComponentSigmaOperator, component_eom_context,
                           component_eom_sources, eom_ccsd_problem)
    from .static import ComponentStaticProblem, component_static_residual, solve_component_ccsd

    if not (hasattr(grid, "upper_shifts") and hasattr(grid, "from_upper") and hasattr(grid, "iw")):
        raise TypeError("grid must be a MatsubaraGrid")
    if rank not in ("S13", "S135"):
        raise ValueError("rank must be 'S13' or 'S135'")
    static = ComponentStaticProblem.compile(model)
    physical = physical_model(static.spec) if static.spec.has_model else physical_model(static.oracle.model)
    block = impurity_sites(physical, sites)
    if amplitudes is None:
        solution = solve_component_ccsd(static, policy=policy, precision=precision)
        if not solution.converged:
            raise RuntimeError(f"static CCSD did not converge (residual {solution.packed_residual_norm:.3e})")
        converged = np.asarray(solution.amplitudes, dtype=np.complex128)
        static_residual = float(solution.packed_residual_norm)
    else:
        converged = np.asarray(amplitudes, dtype=np.complex128)
        retained = component_static_residual(static, converged).retained
        static_residual = float(np.linalg.norm(static.pack(retained)))
    eom = eom_ccsd_problem(static, response_spin=response_spin)
    context = component_eom_context(ComponentEOMProblem.compile(eom, static, 1), converged)
    sources = tuple(component_eom_sources(context, site=site) for site in block)
    if rank == "S13":
        operator = ComponentSigmaOperator(context)
    else:
        from .s135 import CompiledFullS135Action, FullS135ResponseOperator

        operator = FullS135ResponseOperator(CompiledFullS135Action(context))
    response = component_matsubara_green(operator, sources, grid,
                                         maximum_krylov_dimension=maximum_krylov_dimension,
                                         residual_tolerance=residual_tolerance,
                                         minimum_krylov_dimension=minimum_krylov_dimension,
                                         check_interval=check_interval)
    terms = matsubara_self_energy(physical, grid, response.green, sites=block)
    return MatsubaraImpuritySolution(grid=grid, sites=block, rank=rank, response_spin=int(response_spin),
                                     green=response.green, self_energy=terms.self_energy,
                                     noninteracting=terms.noninteracting, hybridization=terms.hybridization,
                                     one_body=terms.one_body, amplitudes=converged, static_residual=static_residual,
                                     response=response, dyson_terms=terms)
