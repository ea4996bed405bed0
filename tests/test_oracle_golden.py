"""Pin the CPU oracle against golden vectors produced by the reference itself."""

from __future__ import annotations

import numpy as np
import pytest

from conftest import GOLDEN as GOLDEN_DIR, eom_amplitudes, golden_names, load, relerr
from oracle import component_oracle as oc


@pytest.mark.parametrize("name", golden_names())
def test_oracle_coordinates_and_tilde_match_reference(name):
    spec, g = load(name)
    p = oc.OracleProblem(spec.as_dict())
    if "cluster_masks" in g:
        assert np.array_equal(np.asarray(p.masks, np.int64), g["cluster_masks"])
    assert np.array_equal(p.tilde.partner, g["tilde_partner"])
    assert np.allclose(p.tilde.phase, g["tilde_phase"], atol=1e-14)
    assert list(p.tilde.independent) == list(g["tilde_independent"])
    assert np.allclose(p.tilde.unpack(g["fixed_variables"]), g["fixed_amplitudes"], atol=1e-18, rtol=0)


@pytest.mark.parametrize("name", golden_names())
def test_oracle_residual_and_jvp_match_reference(name):
    spec, g = load(name)
    p = oc.OracleProblem(spec.as_dict())
    r, ref = p.residual(g["fixed_amplitudes"])
    assert relerr(r, g["residual"]) < 1e-12
    assert abs(ref - g["residual_reference"]) < 1e-12 * max(1.0, abs(g["residual_reference"]))
    j, jref = p.jvp(g["fixed_amplitudes"], g["fixed_direction"])
    assert relerr(j, g["jvp"]) < 1e-12
    assert abs(jref - g["jvp_reference"]) < 1e-12 * max(1.0, abs(g["jvp_reference"]))


@pytest.mark.parametrize("name", golden_names(with_eom=True))
@pytest.mark.parametrize("charge", [1, -1])
def test_oracle_sigma_and_sources_match_reference(name, charge):
    spec, g = load(name)
    tag = "p" if charge == 1 else "m"
    p = oc.OracleProblem(spec.as_dict())
    eom = oc.OracleEOM(p, eom_amplitudes(g), 0, charge)
    if "eom_masks" in g:
        assert np.array_equal(np.asarray(oc.eom_masks(spec.n, 0, charge), np.int64), g["eom_masks"][g[f"eom{tag}_positions"]])
    assert relerr(eom.diagonal, g[f"eom{tag}_diagonal"]) < 1e-14
    assert relerr(eom.sigma(g[f"eom{tag}_probe"]), g[f"eom{tag}_sigma"]) < 1e-12
    add, rem, sink = eom.sources(spec.impurity_site)
    assert np.max(np.abs(add - g[f"eom{tag}_addition"])) < 1e-12
    assert np.max(np.abs(rem - g[f"eom{tag}_removal"])) < 1e-12
    assert np.max(np.abs(sink - g[f"eom{tag}_sink"])) < 1e-14


@pytest.mark.parametrize("name", [n for n in golden_names(with_green=True) if n in ("readme", "s135fix", "twosrc")])
def test_oracle_green_matches_reference_gmres(name):
    spec, g = load(name)
    p = oc.OracleProblem(spec.as_dict())
    eom = oc.OracleEOM(p, g["solution_amplitudes"], 0, 1)
    _, _, gr = oc.retarded_green_dense(eom, spec.impurity_site, g["green_omega"], float(g["green_eta"]))
    assert relerr(gr, g["green_retarded"]) < 1e-8


def test_single_mode_known_answer():
    """G^R of a bare single mode is 1/(omega - eps + i gamma) (reference tests/cc/test_charge_small_sectors.py:17-38).

    Here a one-site spec with one quadratic mode pair and no products checks the
    oracle's sigma/source/sink conventions: sigma is the bare rapidity
    diagonal, and the addition channel resolvent is 1/(z - lambda).
    """
    n = 1
    lam = np.array([0.3 - 1.1j, -0.3 - 1.1j, 0.2 - 0.5j, -0.2 - 0.5j])
    cre = np.zeros((1, 4), complex)
    ann = np.zeros((1, 4), complex)
    cre[0, 0] = 1.0
    ann[0, 1] = 1.0
    spec = dict(n=n, creators=cre, annihilators=ann, product_coefficients=np.zeros(0, complex),
                product_factors=np.zeros((0, 1), np.int64), product_lengths=np.zeros(0, np.int64), rapidities=lam,
                mode_partner=np.array([1, 0, 3, 2]), mode_phase=np.ones(4, complex),
                source_factor=np.zeros((1, 2, 4), np.int64))
    p = oc.OracleProblem(spec)
    eom = oc.OracleEOM(p, np.zeros(p.coords.dimension, complex), 0, 1)
    # S1: one mode; S3: the (1,0,1,1) string; no products -> bare diagonal
    assert eom.dimension == 2
    A = oc.dense_matrix(eom)
    assert np.allclose(A, np.diag([lam[0], lam[0] + lam[2] + lam[3]]))
    w = np.linspace(-2, 2, 9)
    src = eom.source(0)
    sink = np.array([1.0, 0.0])
    g = np.array([sink @ np.linalg.solve(x * np.eye(2) - A, src) for x in w])
    assert np.allclose(g, 1.0 / (w - 0.3 + 1.1j), atol=1e-12)


@pytest.mark.parametrize("name", ["twosrc", "siam10"])
def test_oracle_response_drivers_match_reference(name):
    """Dense forms of the reference's other response drivers (GMRES matrix
    response, complex shifts, Matsubara grid, time propagation) against the
    reference's own outputs on the converged amplitudes, charge +1 (the
    fixtures of ``make_fixtures.py drivers``).  siam10 (EOM dimension 1,947)
    checks the frequency-domain drivers on every fourth shift; its 160-vector
    time-domain bases did not converge in the reference, so only twosrc
    checks the propagators."""
    import c3lindblad_gb300 as c3
    from conftest import GOLDEN

    spec, g = load(name)
    d = np.load(GOLDEN / f"{name}.drivers.npz")
    eom = oc.OracleEOM(oc.OracleProblem(spec.as_dict()), eom_amplitudes(g), 0, 1)
    sites = [int(s) for s in d["sites"]]
    ga, gr = oc.matrix_green_dense(eom, sites, d["gmres_omega"] + 1j * float(d["gmres_eta"]))
    assert relerr(ga, d["gmres_addition"]) < 1e-10
    assert relerr(ga + gr, d["gmres_retarded"]) < 1e-10
    every = 1 if eom.dimension <= 100 else 4
    sa, sr = oc.matrix_green_dense(eom, sites, d["shifts"][::every])
    assert relerr(sa, d["shifts_addition"][::every]) < 1e-10
    assert relerr(sr, d["shifts_removal"][::every]) < 1e-10
    grid = c3.matsubara_grid(float(d["matsubara_beta"]), indices=d["matsubara_indices"])
    upper = grid.upper_shifts[::every]
    ma, mr = oc.matrix_green_dense(eom, sites, upper)
    if every == 1:
        assert relerr(grid.from_upper(ma + mr), d["matsubara_green"]) < 1e-10
    else:  # the grid points n >= 0 of the checked shifts
        pos = [int(np.flatnonzero((grid.indices >= 0) & (2 * grid.indices + 1 == round(z.imag * grid.beta / np.pi)))[0])
               for z in upper]
        assert relerr(ma + mr, d["matsubara_green"][pos]) < 1e-10
    if eom.dimension <= 100:
        comb, add, rem = oc.matrix_time_dense(eom, sites, d["time"])
        assert relerr(comb[:, 0, 0], d["time_retarded"]) < 1e-10
        assert relerr(comb, d["mtime_retarded"]) < 1e-10
        assert relerr(add, d["mtime_addition"]) < 1e-10
        assert relerr(rem, d["mtime_removal"]) < 1e-10


def test_oracle_green_matches_reference_on_the_ed_check_grid():
    """The README model's G^R (eta = 0.1, 161 omega) against the reference's
    CCSD-EOM values of its exact-diagonalisation check, and that check's own
    CCSD-vs-ED deviation (the truncation error, 7.7e-3 relative)."""
    spec, g = load("readme")
    ed = np.load(GOLDEN_DIR / "readme.ed.npz")
    p = oc.OracleProblem(spec.as_dict())
    eom = oc.OracleEOM(p, g["solution_amplitudes"], 0, 1)
    _, _, gr = oc.retarded_green_dense(eom, spec.impurity_site, ed["omega"], float(ed["eta"]))
    assert relerr(gr, ed["green_cc_reference"]) < 1e-8
    dev = relerr(gr, ed["green_ed"])
    assert abs(dev - float(ed["cc_vs_ed_relative"])) <= 1e-7
