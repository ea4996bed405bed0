"""``solve_matsubara`` and the Matsubara self-energy / Dyson steps against the
reference's own ``solve_matsubara`` (``src/c3l/matsubara/solver.py:100``,
``src/c3l/matsubara/dyson.py``).

The goldens (``*.matsubara.npz``, written by ``make_fixtures.py matsubara``)
hold the reference's G(i omega_n), Sigma, G0, the PM hybridization and the
Dyson re-insertion into a semicircular target bath, for both response spins
(and, for the README model, through the S135 response space too), at the
fixture's fixed amplitudes.  The CPU tests feed the reference's G into
the package's host algebra; the GPU tests run the whole device path.  The
conditions mirror the reference's ``tests/test_matsubara.py:135-220``.
"""

from __future__ import annotations

import numpy as np
import pytest

from conftest import GOLDEN, eom_amplitudes, relerr

NAMES = [p.name[: -len(".matsubara.npz")] for p in sorted(GOLDEN.glob("*.matsubara.npz"))]


def _case(name):
    import c3lindblad_gb300 as c3

    ref = dict(np.load(GOLDEN / f"{name}.matsubara.npz"))
    ref["amplitudes"] = eom_amplitudes(np.load(GOLDEN / f"{name}.golden.npz"))
    spec = c3.ProblemSpec.load(GOLDEN / f"{name}.spec.npz")
    grid = c3.matsubara_grid(float(ref["beta"]), indices=ref["indices"])
    return c3, ref, spec, grid


def _tags(ref):
    """(rank, key prefix) of every response the golden holds."""
    out = [("S13", f"s{spin}") for spin in (0, 1)]
    out += [("S135", f"s{spin}_S135") for spin in (0, 1) if f"s{spin}_S135_green" in ref]
    return out


@pytest.mark.parametrize("name", NAMES)
def test_host_self_energy_and_dyson_match_reference(name):
    c3, ref, spec, grid = _case(name)
    sites = tuple(int(s) for s in ref["sites"])
    assert c3.impurity_sites(spec) == sites
    for _, k in _tags(ref):
        terms = c3.matsubara_self_energy(spec, grid, ref[f"{k}_green"])
        assert relerr(terms.noninteracting, ref[f"{k}_noninteracting"]) < 1e-13
        assert relerr(terms.hybridization, ref[f"{k}_hybridization"]) < 1e-12
        assert relerr(terms.self_energy, ref[f"{k}_self_energy"]) < 1e-11
        assert np.allclose(terms.one_body, ref["one_body"], rtol=0, atol=1e-15)
        m = len(sites)
        target = np.broadcast_to(ref["dyson_target_hybridization"][:, None, None] * np.eye(m), terms.hybridization.shape)
        dyson = c3.matsubara_dyson_green(grid, terms.one_body, target, terms.self_energy)
        assert relerr(dyson, ref[f"{k}_dyson_target"]) < 1e-11
        # with the PM hybridization the Dyson equation returns G itself
        back = c3.matsubara_dyson_green(grid, terms.one_body, terms.hybridization, terms.self_energy)
        assert relerr(back, ref[f"{k}_green"]) < 1e-10


def test_self_energy_requires_every_interacting_site():
    import c3lindblad_gb300 as c3

    spec = c3.ProblemSpec.load(GOLDEN / "kanamori3x2.spec.npz")
    grid = c3.matsubara_grid(8.0, n_iw=2)
    green = c3.matsubara_noninteracting_green(spec, grid, (0, 1, 2))
    with pytest.raises(ValueError, match="interaction site"):
        c3.matsubara_self_energy(spec, grid, green[:, :1, :1], sites=(0,))
    with pytest.raises(ValueError, match="shape"):
        c3.matsubara_self_energy(spec, grid, green[:, :1, :1], sites=(0, 1, 2))
    with pytest.raises(ValueError, match="unique"):
        c3.impurity_sites(spec, (0, 1, 2, 2))


def test_noninteracting_green_is_the_pm_resolvent():
    """For one bath site: G0 = 1 / (z - e_d - V^2 / (z - e_b + i Lambda_b))."""
    import c3lindblad_gb300 as c3

    E = np.array([[-0.2, 0.17], [0.17, 0.11]], complex)
    model = c3.PhysicalModel(E, np.diag([0.0, 0.32]).astype(complex), np.diag([0.0, 0.18]).astype(complex), (0,), True)
    grid = c3.matsubara_grid(10.0, n_iw=4)
    z = grid.iw
    delta = 0.17 ** 2 / (np.abs(z.imag) * 1j - 0.11 + 0.5j)
    delta = np.where(grid.indices >= 0, delta, delta.conj())
    G0 = c3.matsubara_noninteracting_green(model, grid)
    assert np.allclose(G0[:, 0, 0], 1.0 / (z + 0.2 - delta), rtol=0, atol=1e-13)
    terms = c3.matsubara_self_energy(model, grid, G0)
    assert np.allclose(terms.self_energy, 0.0, atol=1e-12)
    assert np.allclose(terms.hybridization[:, 0, 0], delta, rtol=0, atol=1e-13)


def test_spec_without_model_is_rejected():
    import dataclasses

    import c3lindblad_gb300 as c3

    spec = c3.ProblemSpec.load(GOLDEN / "readme.spec.npz")
    bare = dataclasses.replace(spec, model_E=None, model_gamma_loss=None, model_gamma_gain=None,
                               interaction_sites=None)
    with pytest.raises(ValueError, match="physical model"):
        c3.physical_model(bare)


@pytest.mark.gpu
@pytest.mark.parametrize("name", NAMES)
def test_solve_matsubara_matches_reference(name, cuda_device):
    c3, ref, spec, grid = _case(name)
    problem = c3.ComponentStaticProblem.compile(spec, device=cuda_device)
    for rank, k in _tags(ref):
        spin = int(k[1])
        sol = c3.solve_matsubara(problem, grid, amplitudes=ref["amplitudes"], response_spin=spin, rank=rank)
        assert sol.sites == tuple(int(s) for s in ref["sites"]) and sol.rank == rank
        assert sol.green.shape == ref[f"{k}_green"].shape
        assert relerr(sol.green, ref[f"{k}_green"]) < 1e-8
        assert relerr(sol.self_energy, ref[f"{k}_self_energy"]) < 1e-7
        assert relerr(sol.noninteracting, ref[f"{k}_noninteracting"]) < 1e-13
        assert abs(sol.static_residual - float(ref["static_residual"])) <= 1e-8 * max(1.0, float(ref["static_residual"]))
        # G(-i w) = G(i w)^dagger carries over to the self-energy
        neg = {int(i): j for j, i in enumerate(grid.indices)}
        for j, i in enumerate(grid.indices):
            jj = neg.get(-int(i) - 1)
            if jj is not None:
                assert np.allclose(sol.self_energy[j], sol.self_energy[jj].conj().T, rtol=0,
                                   atol=1e-9 * np.max(np.abs(sol.self_energy)))
        m = len(sol.sites)
        target = np.broadcast_to(ref["dyson_target_hybridization"][:, None, None] * np.eye(m), sol.hybridization.shape)
        assert relerr(sol.dyson(target), ref[f"{k}_dyson_target"]) < 1e-7


@pytest.mark.gpu
def test_solve_matsubara_rejects_unknown_rank(cuda_device):
    c3, ref, spec, grid = _case(NAMES[0])
    with pytest.raises(ValueError, match="rank"):
        c3.solve_matsubara(c3.ComponentStaticProblem.compile(spec, device=cuda_device), grid,
                           amplitudes=ref["amplitudes"], rank="S15")
