"""Self-energy and Dyson reconstruction of the impurity spectra (host).

Counterparts of ``src/c3l/spectra/reconstruction.py``: the auxiliary
(pseudomode) self-energy from G^R, its re-insertion into another bath, and the
diagnostics the reference reports with them.  They act on the small impurity
block at every frequency, so they run on the host as batched NumPy linear
algebra over the frequency axis (one ``solve``/``cond``/``eigvalsh`` call per
quantity instead of a Python loop over frequencies); the numbers follow the
reference's formulas, which the tests check against the reference's outputs.
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np

_TINY = np.finfo(np.float64).tiny


def _grid(value, name: str) -> np.ndarray:
    a = np.asarray(value, dtype=np.float64)
    if a.ndim != 1 or a.size == 0 or not np.all(np.isfinite(a)):
        raise ValueError(f"{name} must be a finite nonempty one-dimensional array")
    return a


def _vector(value, shape, name: str) -> np.ndarray:
    a = np.asarray(value, dtype=np.complex128)
    if a.shape != shape or not np.all(np.isfinite(a)):
        raise ValueError(f"{name} must be a finite complex vector on omega")
    return a


def _matrices(value, name: str) -> np.ndarray:
    a = np.asarray(value, dtype=np.complex128)
    if a.ndim != 3 or 0 in a.shape or a.shape[1] != a.shape[2] or not np.all(np.isfinite(a)):
        raise ValueError(f"{name} must have finite shape (n_omega,n,n)")
    return a


def _fro(a: np.ndarray) -> np.ndarray:
    return np.linalg.norm(a, ord="fro", axis=(1, 2))


def _spec2(a: np.ndarray) -> np.ndarray:
    return np.linalg.norm(a, ord=2, axis=(1, 2))


@dataclass(frozen=True)
class MatrixResolventDiagnostics:
    """Condition numbers and two-sided backward residuals of ``A G = I`` per frequency."""

    condition_number: np.ndarray
    right_backward_residual: np.ndarray
    left_backward_residual: np.ndarray
    conditioning_limited: np.ndarray
    conditioning_limit: float


@dataclass(frozen=True)
class MatrixSpectralDiagnostics:
    """A = i (G - G^dagger) / 2 pi and its Hermiticity and positivity per frequency."""

    spectral: np.ndarray
    hermiticity_defect: np.ndarray
    minimum_eigenvalue: np.ndarray
    maximum_eigenvalue: np.ndarray
    negative_ratio: np.ndarray


@dataclass(frozen=True)
class MatrixSelfEnergyResult:
    """Sigma = G0^-1 - G^-1 with the conditioning of both inversions."""

    retarded: np.ndarray
    G0_condition_number: np.ndarray
    G_condition_number: np.ndarray
    conditioning_limited: np.ndarray
    dyson: MatrixResolventDiagnostics | None = None


@dataclass(frozen=True)
class MatrixDysonResult:
    inverse_retarded: np.ndarray
    retarded: np.ndarray
    resolvent: MatrixResolventDiagnostics
    spectral: MatrixSpectralDiagnostics


@dataclass(frozen=True)
class MatrixOrderedReconstruction:
    """The PM bath replaced by another one, solved in both resolvent orders."""

    retarded: np.ndarray
    retarded_from_right_order: np.ndarray
    left_ordered_residual: np.ndarray
    right_ordered_residual: np.ndarray
    left_resolvent_identity_residual: np.ndarray
    right_resolvent_identity_residual: np.ndarray
    ordering_difference: np.ndarray
    left_operator_condition_number: np.ndarray
    right_operator_condition_number: np.ndarray
    conditioning_limited: np.ndarray
    spectral: MatrixSpectralDiagnostics


@dataclass(frozen=True)
class PhysicalDysonResult:
    """Scalar physical impurity Green function from the auxiliary self-energy."""

    omega: np.ndarray
    retarded: np.ndarray
    keldysh: np.ndarray
    spectral: np.ndarray


def matrix_resolvent_diagnostics(inverse_green, green, *, conditioning_limit: float = 1.0e10
                                 ) -> MatrixResolventDiagnostics:
    """cond(A) and the backward residuals ||A G - I|| and ||G A - I|| over
    ||A||_2 ||G||_F + ||I||_F (``reconstruction.py:106-142``)."""
    A = _matrices(inverse_green, "inverse_green")
    G = _matrices(green, "green")
    if G.shape != A.shape:
        raise ValueError("inverse_green and green must have the same shape")
    limit = float(conditioning_limit)
    if not np.isfinite(limit) or limit <= 1.0:
        raise ValueError("conditioning_limit must be finite and larger than one")
    eye = np.eye(A.shape[1], dtype=np.complex128)
    denom = _spec2(A) * _fro(G) + np.sqrt(A.shape[1])
    cond = np.linalg.cond(A, p=2)
    return MatrixResolventDiagnostics(cond, _fro(A @ G - eye) / denom, _fro(G @ A - eye) / denom, cond > limit, limit)


def matrix_spectral_diagnostics(G_R) -> MatrixSpectralDiagnostics:
    """The matrix spectral function and its positivity (``reconstruction.py:145-171``)."""
    G = _matrices(G_R, "G_R")
    A = 1j * (G - G.conj().swapaxes(1, 2)) / (2.0 * np.pi)
    herm = _fro(A - A.conj().swapaxes(1, 2)) / np.maximum(_fro(A), _TINY)
    ev = np.linalg.eigvalsh((A + A.conj().swapaxes(1, 2)) / 2.0)
    lo, hi = ev[:, 0], ev[:, -1]
    return MatrixSpectralDiagnostics(A, herm, lo, hi, np.maximum(0.0, -lo) / np.maximum(hi, 1.0e-14))


def matrix_auxiliary_self_energy(G0_R, G_R, *, conditioning_limit: float = 1.0e10) -> MatrixSelfEnergyResult:
    """Sigma = G0^-1 - G^-1 by ordered linear solves (``reconstruction.py:174-212``)."""
    G0 = _matrices(G0_R, "G0_R")
    G = _matrices(G_R, "G_R")
    if G.shape != G0.shape:
        raise ValueError("G0_R and G_R must have the same shape")
    limit = float(conditioning_limit)
    if not np.isfinite(limit) or limit <= 1.0:
        raise ValueError("conditioning_limit must be finite and larger than one")
    eye = np.broadcast_to(np.eye(G.shape[1], dtype=np.complex128), G.shape)
    c0, c = np.linalg.cond(G0, p=2), np.linalg.cond(G, p=2)
    inv0 = np.linalg.solve(G0, eye)
    sigma = inv0 - np.linalg.solve(G, eye)
    dyson = matrix_resolvent_diagnostics(inv0 - sigma, G, conditioning_limit=limit)
    return MatrixSelfEnergyResult(sigma, c0, c, (c0 > limit) | (c > limit), dyson)


def matrix_dyson_green(z, h, Delta_R, Sigma_R, *, conditioning_limit: float = 1.0e10) -> MatrixDysonResult:
    """G = [z I - h - Delta - Sigma]^-1 on a frequency grid (``reconstruction.py:215-257``)."""
    shifts = np.asarray(z, dtype=np.complex128)
    delta = _matrices(Delta_R, "Delta_R")
    sigma = _matrices(Sigma_R, "Sigma_R")
    one = np.asarray(h, dtype=np.complex128)
    m = delta.shape[1]
    if (shifts.shape != (delta.shape[0],) or not np.all(np.isfinite(shifts)) or sigma.shape != delta.shape
            or one.shape != (m, m) or not np.all(np.isfinite(one))):
        raise ValueError("z, h, Delta_R, and Sigma_R have incompatible shapes")
    eye = np.eye(m, dtype=np.complex128)
    lhs = shifts[:, None, None] * eye[None] - one[None] - delta - sigma
    green = np.linalg.solve(lhs, np.broadcast_to(eye, lhs.shape))
    return MatrixDysonResult(lhs, green, matrix_resolvent_diagnostics(lhs, green, conditioning_limit=conditioning_limit),
                             matrix_spectral_diagnostics(green))


def matrix_ordered_dyson_reconstruction(G_PM_R, Delta_PM_R, Delta_physical_R, *,
                                        conditioning_limit: float = 1.0e10) -> MatrixOrderedReconstruction:
    """Replace the PM bath by the physical one: (I - G_PM D) G = G_PM and
    G (I - D G_PM) = G_PM with D = Delta_physical - Delta_PM, both solved and
    their resolvent identities re-applied (``reconstruction.py:260-356``)."""
    Gp = _matrices(G_PM_R, "G_PM_R")
    dpm = _matrices(Delta_PM_R, "Delta_PM_R")
    dph = _matrices(Delta_physical_R, "Delta_physical_R")
    if dpm.shape != Gp.shape or dph.shape != Gp.shape:
        raise ValueError("all reconstruction arrays must have the same shape")
    eye = np.eye(Gp.shape[1], dtype=np.complex128)
    D = dph - dpm
    left_op = eye - Gp @ D
    right_op = eye - D @ Gp
    left = np.linalg.solve(left_op, Gp)
    right = np.linalg.solve(right_op.swapaxes(1, 2), Gp.swapaxes(1, 2)).swapaxes(1, 2)
    gpf = _fro(Gp)
    l_res = _fro(left_op @ left - Gp) / (_spec2(left_op) * _fro(left) + gpf)
    r_res = _fro(right @ right_op - Gp) / (_spec2(right_op) * _fro(right) + gpf)
    change = left - Gp
    lp = Gp @ D @ left
    rp = left @ D @ Gp
    l_id = _fro(change - lp) / np.maximum(_fro(change) + _fro(lp), _TINY)
    r_id = _fro(change - rp) / np.maximum(_fro(change) + _fro(rp), _TINY)
    diff = _fro(left - right) / np.maximum(_fro(left), _TINY)
    lc, rc = np.linalg.cond(left_op, p=2), np.linalg.cond(right_op, p=2)
    limit = float(conditioning_limit)
    return MatrixOrderedReconstruction(left, right, l_res, r_res, l_id, r_id, diff, lc, rc, (lc > limit) | (rc > limit),
                                       matrix_spectral_diagnostics(left))


def noninteracting_auxiliary_green(model, omega, *, eta: float = 0.0) -> tuple[np.ndarray, np.ndarray]:
    """Impurity G0^R and G0^K of the Lindblad one-body model
    (``reconstruction.py:359-394``): G^R = (w + i eta - E + i Lambda)^-1,
    G^K = 2i G^R Omega G^A with Lambda = loss + gain, Omega = gain - loss."""
    from .matsubara import physical_model

    m = physical_model(model)
    w = _grid(omega, "omega")
    b = float(eta)
    if not np.isfinite(b) or b < 0.0:
        raise ValueError("eta must be finite and nonnegative")
    eye = np.eye(m.n_sites, dtype=np.complex128)
    lam = m.gamma_loss + m.gamma_gain
    om = m.gamma_gain - m.gamma_loss
    GR = np.linalg.inv((w + 1j * b)[:, None, None] * eye[None] - m.E[None] + 1j * lam[None])
    GK = 2j * GR @ om[None] @ GR.conj().swapaxes(1, 2)
    f = m.impurity_site
    return np.ascontiguousarray(GR[:, f, f]), np.ascontiguousarray(GK[:, f, f])


def auxiliary_self_energy(G0_R, G0_K, G_R, G_K) -> tuple[np.ndarray, np.ndarray]:
    """Scalar Sigma^R = 1/G0^R - 1/G^R and Sigma^K = -G0^K/|G0^R|^2 + G^K/|G^R|^2
    (``reconstruction.py:397-423``)."""
    g0r = np.asarray(G0_R, dtype=np.complex128)
    if g0r.ndim != 1 or g0r.size == 0:
        raise ValueError("G0_R must be a nonempty vector")
    g0k = _vector(G0_K, g0r.shape, "G0_K")
    gr = _vector(G_R, g0r.shape, "G_R")
    gk = _vector(G_K, g0r.shape, "G_K")
    if not np.all(np.isfinite(g0r)):
        raise ValueError("G0_R must be finite")
    if np.any(np.abs(g0r) <= _TINY) or np.any(np.abs(gr) <= _TINY):
        raise ValueError("Green function has a zero that makes Sigma undefined")
    return 1.0 / g0r - 1.0 / gr, -g0k / np.abs(g0r) ** 2 + gk / np.abs(gr) ** 2


def physical_dyson_reconstruction(omega, epsilon_imp: float, Delta_R, Delta_K, Sigma_R, Sigma_K
                                  ) -> PhysicalDysonResult:
    """G^R = 1/(w - eps - Delta^R - Sigma^R), G^K = |G^R|^2 (Delta^K + Sigma^K)
    (``reconstruction.py:448-473``)."""
    w = _grid(omega, "omega")
    eps = float(epsilon_imp)
    if not np.isfinite(eps):
        raise ValueError("epsilon_imp must be finite")
    dr, dk = _vector(Delta_R, w.shape, "Delta_R"), _vector(Delta_K, w.shape, "Delta_K")
    sr, sk = _vector(Sigma_R, w.shape, "Sigma_R"), _vector(Sigma_K, w.shape, "Sigma_K")
    den = w - eps - dr - sr
    if np.any(np.abs(den) <= _TINY):
        raise ValueError("physical Dyson denominator vanishes on the grid")
    gr = 1.0 / den
    return PhysicalDysonResult(w, gr, np.abs(gr) ** 2 * (dk + sk), -gr.imag / np.pi)


def equilibrium_fdt_defect(omega, G_R, G_K, temperature: float) -> float:
    """Relative defect of G^K = (G^R - G^A) tanh(w / 2T) (``reconstruction.py:476-492``)."""
    w = _grid(omega, "omega")
    gr, gk = _vector(G_R, w.shape, "G_R"), _vector(G_K, w.shape, "G_K")
    T = float(temperature)
    if not np.isfinite(T) or T <= 0.0:
        raise ValueError("temperature must be finite and positive")
    want = (gr - gr.conj()) * np.tanh(w / (2.0 * T))
    return float(np.linalg.norm(gk - want) / max(float(np.linalg.norm(want)), _TINY))


def particle_hole_spectral_defect(omega, spectral) -> float:
    """max |A(w) - A(-w)| / max |A| on a symmetric grid (``reconstruction.py:495-505``)."""
    w = _grid(omega, "omega")
    A = np.asarray(spectral, dtype=np.float64)
    if A.shape != w.shape or not np.all(np.isfinite(A)):
        raise ValueError("spectral must be a finite vector on omega")
    if not np.allclose(w, -w[::-1], atol=2.0e-14, rtol=2.0e-14):
        raise ValueError("particle-hole diagnostic requires a symmetric grid")
    return float(np.max(np.abs(A - A[::-1])) / max(float(np.max(np.abs(A))), _TINY))


def spectral_grid_diagnostics(omega, G_R) -> dict:
    """Causality, the finite-grid sum rule and the high-frequency moment
    (``reconstruction.py:508-532``)."""
    w = _grid(omega, "omega")
    gr = _vector(G_R, w.shape, "G_R")
    A = -gr.imag / np.pi
    order = np.argsort(w)
    total = float(np.trapezoid(A[order], x=w[order]))
    edge = max(1, min(4, w.size // 4))
    far = np.argsort(np.abs(w))[-edge:]
    return {"minimum_spectral_weight": float(np.min(A)), "causality_violation": float(max(0.0, np.max(gr.imag))),
            "finite_grid_sum": total, "finite_grid_sum_rule_defect": abs(total - 1.0),
            "high_frequency_moment_defect": float(np.max(np.abs(w[far] * gr[far] - 1.0)))}


__all__ = [
    "MatrixDysonResult", "MatrixOrderedReconstruction", "MatrixResolventDiagnostics", "MatrixSelfEnergyResult",
    "MatrixSpectralDiagnostics", "PhysicalDysonResult", "auxiliary_self_energy", "equilibrium_fdt_defect",
    "matrix_auxiliary_self_energy", "matrix_dyson_green", "matrix_ordered_dyson_reconstruction",
    "matrix_resolvent_diagnostics", "matrix_spectral_diagnostics", "noninteracting_auxiliary_green",
    "particle_hole_spectral_defect", "physical_dyson_reconstruction", "spectral_grid_diagnostics",
]
