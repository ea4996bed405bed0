"""Host-side logic of the response drivers (no GPU): argument checks that the
reference's drivers make before any action (``src/c3l/cc/component_response.py``)
and the reduced time propagation of an Arnoldi projection
(``src/c3l/green/krylov.py:134-208``), checked against a direct matrix
exponential."""

from __future__ import annotations

from types import SimpleNamespace

import numpy as np
import pytest

torch = pytest.importorskip("torch")
scipy_linalg = pytest.importorskip("scipy.linalg")

import c3lindblad_gb300 as c3  # noqa: E402
from c3lindblad_gb300.response import ArnoldiProjection  # noqa: E402


def _sources(count: int, dim: int, *, charge: int = 1):
    rng = np.random.default_rng(5)
    out = []
    for site in range(count):
        v = [rng.normal(size=dim) + 1j * rng.normal(size=dim) for _ in range(3)]
        out.append(c3.ComponentEOMSources(v[0], v[1], v[2], charge, site))
    return out


def _operator(dim: int):
    return SimpleNamespace(dimension=dim, action_calls=0, action_wall_seconds=0.0)


def test_shifted_matrix_driver_rejects_bad_shifts_and_sources():
    op = _operator(12)
    with pytest.raises(ValueError, match="positive imaginary"):
        c3.component_retarded_matrix_green_shifts(op, _sources(2, 12), [1.0 + 0.0j])
    with pytest.raises(ValueError, match="positive imaginary"):
        c3.component_retarded_matrix_green_shifts(op, _sources(2, 12), [0.5 + 0.1j, np.nan])
    with pytest.raises(ValueError, match="at least one"):
        c3.component_retarded_matrix_green_shifts(op, [], [1j])
    with pytest.raises(ValueError, match="unique"):
        c3.component_retarded_matrix_green_shifts(op, _sources(1, 12) * 2, [1j])
    with pytest.raises(ValueError, match="smaller"):
        c3.component_retarded_matrix_green_shifts(_operator(8), _sources(2, 12), [1j])
    with pytest.raises(TypeError):
        c3.component_retarded_matrix_green_shifts(SimpleNamespace(dimension=12), _sources(2, 12), [1j])
    with pytest.raises(TypeError):
        c3.component_retarded_matrix_green_shifts(op, _sources(2, 12), [1j], maximum_krylov_dimension=8.5)


def test_time_and_gmres_matrix_drivers_reject_bad_arguments():
    op = _operator(12)
    with pytest.raises(ValueError, match="finite nonempty"):
        c3.component_retarded_matrix_time(op, _sources(2, 12), [0.0, -1.0], [1j])
    with pytest.raises(ValueError, match="finite nonempty"):
        c3.component_retarded_matrix_time(op, _sources(2, 12), [0.0, 1.0], [])
    mixed = _sources(1, 12) + _sources(1, 12, charge=-1)
    mixed[1].site = 1
    with pytest.raises(ValueError, match="one response charge"):
        c3.component_retarded_matrix_time(op, mixed, [0.0], [1j])
    with pytest.raises(ValueError, match="positive eta"):
        c3.component_retarded_matrix_green(op, _sources(2, 12), [0.0, 1.0], 0.0)
    with pytest.raises(ValueError, match="retained basis"):
        bad = _sources(2, 12)
        bad[1].sink = bad[1].sink[:5]
        c3.component_retarded_matrix_green(op, bad, [0.0], 0.1)


def _projection(m: int, N: int, seed: int = 1):
    rng = np.random.default_rng(seed)
    H = np.triu(rng.normal(size=(m + 1, m)) + 1j * rng.normal(size=(m + 1, m)), -1) * 0.3
    H[np.arange(1, m + 1), np.arange(m)] = np.abs(H[np.arange(1, m + 1), np.arange(m)]) + 0.1
    basis = SimpleNamespace(V=torch.zeros((m + 1, N), dtype=torch.complex128), H=H, beta=1.7, breakdown=False,
                            check_dimensions=[m], check_residuals=[1e-3], converged=True, wall_seconds=0.0,
                            residual=None)
    return ArnoldiProjection(basis, 1e-10, 0), H


@pytest.mark.parametrize("grid", ["uniform", "ragged", "single"])
def test_time_coefficients_match_the_matrix_exponential(grid):
    proj, H = _projection(12, 30)
    t = {"uniform": np.linspace(0.0, 3.0, 13), "ragged": np.array([0.0, 0.1, 0.7, 2.5]),
         "single": np.array([1.3])}[grid]
    Y = proj.time_coefficients(t)
    e1 = np.zeros(12, complex)
    e1[0] = 1.7
    want = np.asarray([scipy_linalg.expm(-1j * v * H[:12, :12]) @ e1 for v in t])
    assert np.max(np.abs(Y - want)) <= 1e-12 * max(1.0, np.max(np.abs(want)))
    res = proj.relative_time_residuals(t)
    assert np.allclose(res, np.abs(H[12, 11] * want[:, -1]) / 1.7, rtol=1e-12, atol=1e-15)
    # a saved prefix uses the leading block of H only
    Y6 = proj.time_coefficients(t, dimension=6)
    want6 = np.asarray([scipy_linalg.expm(-1j * v * H[:6, :6]) @ e1[:6] for v in t])
    assert np.max(np.abs(Y6 - want6)) <= 1e-12 * max(1.0, np.max(np.abs(want6)))
    with pytest.raises(ValueError):
        proj.time_coefficients([np.inf])
    with pytest.raises(ValueError):
        proj.time_coefficients(t, dimension=13)


def test_matsubara_grid_maps_upper_values_and_checks_the_lattice():
    grid = c3.matsubara_grid(5.0, n_iw=3)
    assert list(grid.indices) == [-3, -2, -1, 0, 1, 2]
    assert np.allclose(grid.upper_shifts, 1j * np.array([1, 3, 5]) * np.pi / 5.0)
    rng = np.random.default_rng(2)
    upper = rng.normal(size=(3, 2, 2)) + 1j * rng.normal(size=(3, 2, 2))
    full = grid.from_upper(upper)
    # n = -1 and n = 0 share |2n + 1| = 1: G(-i w) = G(i w)^dagger
    assert np.array_equal(full[3], upper[0])
    assert np.array_equal(full[2], upper[0].conj().T)
    assert np.array_equal(full[0], upper[2].conj().T)
    scalar = grid.from_upper(upper[:, 0, 0])
    assert scalar[1] == np.conj(upper[1, 0, 0])
    same = c3.matsubara_grid(5.0, omega_n=grid.iw)
    assert np.array_equal(same.indices, grid.indices)
    with pytest.raises(ValueError, match="fermionic"):
        c3.matsubara_grid(5.0, omega_n=[2 * np.pi / 5.0])
    with pytest.raises(ValueError, match="exactly one"):
        c3.matsubara_grid(5.0, n_iw=2, indices=[0])
    with pytest.raises(ValueError, match="unique"):
        c3.matsubara_grid(5.0, indices=[0, 0])
    with pytest.raises(ValueError, match="shape"):
        grid.from_upper(np.zeros(4))
    with pytest.raises(TypeError):
        c3.component_matsubara_green(_operator(12), _sources(1, 12), object())
