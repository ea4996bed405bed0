"""Spectra reconstruction (``src/c3l/spectra/reconstruction.py``) against the
reference's own outputs on the same inputs (``spectra.reconstruction.npz``,
written by ``make_fixtures.py spectra``): the scalar auxiliary self-energy
and physical Dyson reconstruction on the siam10 CCSD G^R, and the matrix
self-energy, Dyson and ordered reconstruction on the n = 9 Kanamori impurity
block, with their diagnostics."""

from __future__ import annotations

import numpy as np
import pytest

from conftest import GOLDEN, relerr

REF = GOLDEN / "spectra.reconstruction.npz"


@pytest.fixture(scope="module")
def ref():
    return np.load(REF)


def test_scalar_auxiliary_self_energy_and_physical_dyson(ref):
    import c3lindblad_gb300 as c3

    spec = c3.ProblemSpec.load(GOLDEN / "siam10.spec.npz")
    w = ref["scalar_omega"]
    g0r, g0k = c3.noninteracting_auxiliary_green(spec, w, eta=0.05)
    assert relerr(g0r, ref["scalar_G0_R"]) < 1e-13 and relerr(g0k, ref["scalar_G0_K"]) < 1e-13
    sr, sk = c3.auxiliary_self_energy(g0r, g0k, ref["scalar_G_R"], ref["scalar_G_K"])
    assert relerr(sr, ref["scalar_Sigma_R"]) < 1e-12 and relerr(sk, ref["scalar_Sigma_K"]) < 1e-12
    phys = c3.physical_dyson_reconstruction(w, -2.0, ref["scalar_Delta_R"], ref["scalar_Delta_K"], sr, sk)
    for k in ("retarded", "keldysh", "spectral"):
        assert relerr(getattr(phys, k), ref[f"phys_{k}"]) < 1e-12
    assert c3.equilibrium_fdt_defect(w, ref["scalar_G_R"], ref["scalar_G_K"], 0.1) == pytest.approx(
        float(ref["fdt_defect"]), rel=1e-10, abs=1e-15)
    assert c3.particle_hole_spectral_defect(w, -ref["scalar_G_R"].imag / np.pi) == pytest.approx(
        float(ref["ph_defect"]), rel=1e-12)
    diag = c3.spectral_grid_diagnostics(w, ref["scalar_G_R"])
    assert np.allclose(list(diag.values()), ref["grid_diagnostics"], rtol=1e-12, atol=1e-15)
    with pytest.raises(ValueError, match="symmetric"):
        c3.particle_hole_spectral_defect(w + 0.1, -ref["scalar_G_R"].imag)


def test_matrix_self_energy_dyson_and_ordered_reconstruction(ref):
    import c3lindblad_gb300 as c3

    mse = c3.matrix_auxiliary_self_energy(ref["matrix_G0"], ref["matrix_G"])
    assert relerr(mse.retarded, ref["mse_retarded"]) < 1e-12
    assert np.allclose(mse.G0_condition_number, ref["mse_G0_cond"], rtol=1e-10)
    assert np.allclose(mse.G_condition_number, ref["mse_G_cond"], rtol=1e-10)
    # backward residuals are rounding-level quantities: the same order of magnitude
    assert np.all(mse.dyson.right_backward_residual < 1e-14) and np.all(ref["mse_dyson_right"] < 1e-14)
    md = c3.matrix_dyson_green(ref["matrix_z"], ref["matrix_h"], ref["matrix_Delta_phys"], mse.retarded)
    assert relerr(md.retarded, ref["md_retarded"]) < 1e-11
    assert relerr(md.inverse_retarded, ref["md_inverse"]) < 1e-12
    assert np.allclose(md.resolvent.condition_number, ref["md_cond"], rtol=1e-9)
    assert relerr(md.spectral.spectral, ref["md_spectral"]) < 1e-11
    for mine, k in ((md.spectral.minimum_eigenvalue, "md_min_eig"), (md.spectral.maximum_eigenvalue, "md_max_eig")):
        assert np.allclose(mine, ref[k], rtol=1e-9, atol=1e-13)
    assert np.all(md.resolvent.right_backward_residual < 1e-14)
    mo = c3.matrix_ordered_dyson_reconstruction(ref["matrix_G"], ref["matrix_Delta_PM"], ref["matrix_Delta_phys"])
    assert relerr(mo.retarded, ref["mo_retarded"]) < 1e-11
    assert relerr(mo.retarded_from_right_order, ref["mo_right_order"]) < 1e-11
    assert np.allclose(mo.left_operator_condition_number, ref["mo_left_cond"], rtol=1e-9)
    assert np.allclose(mo.right_operator_condition_number, ref["mo_right_cond"], rtol=1e-9)
    for mine, k in ((mo.left_ordered_residual, "mo_left_res"), (mo.ordering_difference, "mo_diff"),
                    (mo.left_resolvent_identity_residual, "mo_left_id")):
        assert np.all(mine < 1e-13) and np.all(ref[k] < 1e-13)
    with pytest.raises(ValueError, match="same shape"):
        c3.matrix_ordered_dyson_reconstruction(ref["matrix_G"], ref["matrix_Delta_PM"][:-1], ref["matrix_Delta_phys"])
