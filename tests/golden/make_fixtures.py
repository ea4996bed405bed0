"""Generate problem specs and golden vectors by running the reference itself.

This script is test infrastructure.  It imports the reference package
(``c3l``) from a source tree given on the command line (default: the
read-only checkout next to this repository), builds each seeded model with the
reference's own setup code, runs the reference's CPU hot path and writes:

* ``<name>.spec.npz`` -- the self-contained problem description consumed by
  ``c3lindblad_gb300.spec.ProblemSpec`` (site count, distinct linear factors as
  creator/annihilator vectors over the 4n particle-hole modes, the factorized
  products, rapidities, mode-level tilde partners/phases, source operators);
* ``<name>.golden.npz`` -- reference outputs on that problem: residual and JVP
  at deterministic amplitudes (the fixture recipe of the reference's
  ``tests/cc/test_component_jax.py:41-44``), cluster/EOM masks and tilde maps
  (small n only), the converged Newton--Krylov solution, the EOM diagonal,
  a sigma action, the sources, and G^R on a frequency grid.

The GPU machine never runs this script; only the ``.npz`` files travel.

Usage: ``python tests/golden/make_fixtures.py [--reference SRC] [names...]``;
``... matrix [fixtures...]``, ``... warmstart``, ``... drivers [names...]`` and
``... ed`` write the matrix-response, warm-start, response-driver and
exact-diagonalisation fixtures; ``... spec [names...]`` writes the specs of
``SPEC_ONLY`` (no reference outputs); ``... model [names...]`` adds the
physical one-body model (E, gamma_loss, gamma_gain, interaction sites) to
committed specs; ``... matsubara`` writes the reference's ``solve_matsubara``
outputs; ``... s135 [names...]`` writes the reference's full S135 response
actions; ``... spectra`` the reference's spectra reconstruction outputs;
``... static names...`` the static goldens alone (residual and JVP at the fixed
amplitudes).
"""

from __future__ import annotations

import argparse
import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent


def _import_reference(src: str):
    sys.path.insert(0, src)
    import c3l  # noqa: F401


# ---------------------------------------------------------------- models
def model_readme():
    """README quick-start model (reference README.md)."""
    from c3l import FermionicLindbladModel

    return FermionicLindbladModel(
        E=np.array([[-0.6, 0.28, 0.28], [0.28, -1.2, 0.0], [0.28, 0.0, 1.2]]),
        gamma_loss=np.diag([0.0, 0.06, 0.48]),
        gamma_gain=np.diag([0.0, 0.48, 0.06]),
        U=1.2,
    )


def model_s135():
    """Compact interacting model of the reference tests (tests/s135_fixture.py:8-30)."""
    from c3l import FermionicLindbladModel

    U = 1.2
    bath = np.linspace(-1.2, 1.2, 2)
    E = np.diag(np.concatenate(([-U / 2.0], bath))).astype(np.complex128)
    coupling = 0.28 + 0.04 * (1.0 - np.abs(bath) / np.max(np.abs(bath)))
    E[0, 1:] = coupling
    E[1:, 0] = coupling
    scaled = (bath - bath[0]) / (bath[-1] - bath[0])
    loss = np.zeros(3)
    gain = np.zeros(3)
    loss[1:] = 0.06 + 0.42 * scaled
    gain[1:] = 0.48 - 0.42 * scaled
    return FermionicLindbladModel(E, np.diag(loss), np.diag(gain), U=U)


def model_twosrc():
    """Two-site complex-hopping model (tests/cc/test_component_jax.py:47-58)."""
    from c3l import FermionicLindbladModel

    U = 0.4
    E = np.asarray(((-0.5 * U, 0.18j), (-0.18j, 0.25)))
    return FermionicLindbladModel(E, np.diag((0.0, 0.32)), np.diag((0.0, 0.11)), U=U)


def model_siam(num_modes: int, seed: int):
    """Single-impurity Anderson model with Lindblad pseudomodes (seeded)."""
    from c3l import FermionicLindbladModel

    rng = np.random.default_rng(seed)
    U = 4.0
    eb = rng.uniform(-3, 3, num_modes)
    V = rng.normal(0, 0.3, num_modes)
    r = rng.uniform(0.05, 0.5, num_modes)
    f = 1.0 / (np.exp(eb / 0.1) + 1.0)
    E = np.diag(np.r_[-U / 2, eb]).astype(complex)
    E[0, 1:] = V
    E[1:, 0] = V
    return FermionicLindbladModel(E, np.diag(np.r_[0, r * (1 - f)]), np.diag(np.r_[0, r * f]), U=U)


def model_kanamori(norb: int, modes_per_orbital: int, seed: int):
    """Multi-orbital Kanamori impurity with seeded pseudomode baths."""
    from c3l import FermionicLindbladModel
    from c3l.cc._static_schema import interaction_from_spatial_tensor
    from c3l.interactions import SparseTwoBodyInteraction

    rng = np.random.default_rng(seed)
    U, J = 2.0, 0.3
    Up = U - 2 * J
    K = np.zeros((norb,) * 4)
    for a in range(norb):
        for b in range(norb):
            if a == b:
                K[a, a, a, a] = U / 2
            else:
                K[a, b, a, b] = Up / 2
                K[a, b, b, a] = J / 2
                K[a, a, b, b] = J / 2
    terms = interaction_from_spatial_tensor(K)
    nm = modes_per_orbital
    n = norb * (1 + nm)
    E = np.zeros((n, n), complex)
    loss = np.zeros(n)
    gain = np.zeros(n)
    E[:norb, :norb] = np.diag(rng.uniform(-0.2, 0.2, norb)) - U / 2
    for o in range(norb):
        eb = rng.uniform(-3, 3, nm)
        V = rng.normal(0, 0.3, nm)
        r = rng.uniform(0.05, 0.5, nm)
        f = 1 / (np.exp(eb / 0.1) + 1)
        s = slice(norb + o * nm, norb + (o + 1) * nm)
        E[s, s] = np.diag(eb)
        E[o, s] = V
        E[s, o] = V
        loss[s] = r * (1 - f)
        gain[s] = r * f
    inter = SparseTwoBodyInteraction(2 * n, terms.terms)
    return FermionicLindbladModel(
        E, np.diag(loss), np.diag(gain), U=0.0,
        interaction_sites=tuple(range(norb)), two_body_interaction=inter,
    )


def model_general(norb: int, modes_per_orbital: int, seed: int):
    """General-interaction impurity: ``norb`` orbitals with a seeded Gaussian
    spatial tensor U_abcd (scale 0.5) made Hermitian and permutation-symmetric
    (U_abcd = U_badc = conj(U_dcba)), lowered to spin-orbital terms by the
    reference's ``interaction_from_spatial_tensor`` (``_static_schema.py:77``);
    a GOE impurity one-body block (scale 0.3) and seeded pseudomode baths per
    orbital drawn as for the single-impurity model (T = 0.1, mu = 0)."""
    from c3l import FermionicLindbladModel
    from c3l.cc._static_schema import interaction_from_spatial_tensor
    from c3l.interactions import SparseTwoBodyInteraction

    rng = np.random.default_rng(seed)
    K = rng.normal(0.0, 0.5, (norb,) * 4)
    K = 0.5 * (K + K.transpose(1, 0, 3, 2))
    K = 0.5 * (K + K.transpose(3, 2, 1, 0).conj())
    terms = interaction_from_spatial_tensor(K)
    nm = modes_per_orbital
    n = norb * (1 + nm)
    E = np.zeros((n, n), complex)
    loss = np.zeros(n)
    gain = np.zeros(n)
    A = rng.normal(0.0, 0.3, (norb, norb))
    E[:norb, :norb] = (A + A.T) / np.sqrt(2.0)
    for o in range(norb):
        eb = rng.uniform(-3, 3, nm)
        V = rng.normal(0, 0.3, nm)
        r = rng.uniform(0.05, 0.5, nm)
        f = 1 / (np.exp(eb / 0.1) + 1)
        s = slice(norb + o * nm, norb + (o + 1) * nm)
        E[s, s] = np.diag(eb)
        E[o, s] = V
        E[s, o] = V
        loss[s] = r * (1 - f)
        gain[s] = r * f
    inter = SparseTwoBodyInteraction(2 * n, terms.terms)
    return FermionicLindbladModel(
        E, np.diag(loss), np.diag(gain), U=0.0,
        interaction_sites=tuple(range(norb)), two_body_interaction=inter,
    )


def _restricted_reference(model):
    from c3l.ci.reference import full_hartree_fock_reference
    from c3l.gaussian_mean_field import solve_ghf

    hf = solve_ghf(
        model.physical_E, model.interaction, model.physical_gamma_loss, model.physical_gamma_gain,
        restricted=True, tolerance=1e-10, max_iterations=600, damping=0.5,
        terminal_least_squares=True,
    )
    if not hf.converged:
        raise RuntimeError("restricted GHF reference did not converge")
    return full_hartree_fock_reference(model, hf.fock, hf.gamma)


# name -> (builder, reference recipe, amplitude scale, omega grid, eta, solve?)
FIXTURES = {
    "readme": dict(model=model_readme, recipe="full_hf", scale=7e-4,
                   omega=np.linspace(-4.0, 4.0, 81), eta=0.0, solve=True),
    "s135fix": dict(model=model_s135, recipe="legacy_half_filled:0.3", scale=7e-4,
                    omega=np.linspace(-3.0, 3.0, 25), eta=0.05, solve=True),
    "twosrc": dict(model=model_twosrc, recipe="legacy_half_filled:0.3", scale=5e-4,
                   omega=np.linspace(-2.0, 2.0, 17), eta=0.1, solve=True),
    "siam10": dict(model=lambda: model_siam(10, 0), recipe="legacy_half_filled:0.5", scale=1e-3,
                   omega=np.linspace(-8.0, 8.0, 1001), eta=0.0, solve=True),
    # the reference's Newton solve does not converge on these Kanamori draws from
    # zero amplitudes, so EOM parity uses the fixed amplitudes instead
    "kanamori3x2": dict(model=lambda: model_kanamori(3, 2, 2), recipe="restricted_ghf", scale=1e-3,
                        omega=None, eta=0.02, solve=False, eom=True),
    "kanamori3x8": dict(model=lambda: model_kanamori(3, 8, 2), recipe="restricted_ghf", scale=1e-3,
                        omega=None, eta=0.02, solve=False, eom=True),
    # the general-interaction (5 orbitals, seeded U_abcd) model with one
    # pseudomode per orbital: the product structure of the 12-mode workload
    # (1,650 four-factor products + 100 counterterms over 40 factors) at n = 10.
    # The reference needs 41 s per JVP here, so its own Newton solve is out of
    # reach; the goldens (actions, sources, G^R) are taken at the fixed amplitudes
    "gen5x1": dict(model=lambda: model_general(5, 1, 0), recipe="restricted_ghf", scale=1e-3,
                   omega=np.linspace(-12.0, 12.0, 4096)[::128], eta=0.02, solve=False, eom=True),
}

# specs only (no reference hot-path run): the 12-mode general-interaction model
# (n = 65), built without the cluster masks
SPEC_ONLY = {
    "gen5x12": dict(model=lambda: model_general(5, 12, 0), recipe="restricted_ghf"),
}


def light_problem(model, reference):
    """The fields of the reference's ``FactorizedCCProblem`` that a spec reads
    (model, reference, products, rapidities), built by the reference's own
    product constructors but without the cluster masks and amplitude tilde map
    (``src/c3l/cc/factorized.py:336-414``).  Those are Python loops over every
    amplitude, too slow at n = 65; the package derives both itself.  The
    one-body counterterm loop for an unregulated reference restates
    ``factorized.py:383-414``."""
    from types import SimpleNamespace

    from c3l.cc.factorized import _quadratic_dissipation_counterterms
    from c3l.ci.matrix_free import FactorizedModeProduct, _interaction_products, physical_mode_operator

    products = list(_interaction_products(reference))
    if reference.reference_gamma_loss is not None:
        products.extend(_quadratic_dissipation_counterterms(model, reference))
    else:
        E = np.asarray(model.E)
        blocks = tuple(E - np.asarray(b) for b in reference.one_body_blocks)
        for i in range(model.n_sites):
            for j in range(model.n_sites):
                for spin, delta in enumerate(blocks):
                    if delta[i, j] == 0.0:
                        continue
                    op = lambda site, ch: physical_mode_operator(reference, site, spin, ch)
                    products.append(FactorizedModeProduct(
                        f"quadratic_counter:c_{i}_{spin}_dagger_c_{j}_{spin}", complex(delta[i, j]),
                        (op(i, "c_dagger"), op(j, "c"))))
                    products.append(FactorizedModeProduct(
                        f"quadratic_counter:-tilde_c_{i}_{spin}_dagger_tilde_c_{j}_{spin}", -complex(delta[j, i]),
                        (op(i, "tilde_c_dagger"), op(j, "tilde_c"))))
    rapidities = np.asarray(
        tuple(v for block in reference.mode_references for v in block.rapidities), dtype=np.complex128)
    return SimpleNamespace(model=model, reference=reference, products=tuple(products), rapidities=rapidities)


def build_reference(spec):
    """The HF reference of a fixture recipe (as ``factorized_cc_problem`` builds it)."""
    model = spec["model"]()
    recipe = spec["recipe"]
    if recipe == "restricted_ghf":
        return model, _restricted_reference(model)
    raise ValueError(f"mask-free build supports the restricted GHF recipe only, not {recipe}")


def build_problem(spec):
    from c3l.cc.factorized import factorized_cc_problem

    model = spec["model"]()
    recipe = spec["recipe"]
    if recipe == "full_hf":
        cc = factorized_cc_problem(model, "CCSD")
    elif recipe.startswith("legacy_half_filled"):
        m_up = float(recipe.split(":")[1])
        cc = factorized_cc_problem(model, "CCSD", m_up=m_up, reference_mode="legacy_half_filled")
    elif recipe == "restricted_ghf":
        cc = factorized_cc_problem(model, "CCSD", reference=_restricted_reference(model))
    else:
        raise ValueError(recipe)
    return cc


def export_spec(cc, path: Path, recipe: str) -> dict:
    """Write the self-contained problem description, lowered by the package's
    own ``ProblemSpec.from_factorized`` (the path ``ComponentStaticProblem.compile``
    takes for a reference object)."""
    sys.path.insert(0, str(HERE.parents[1]))
    from c3lindblad_gb300.spec import ProblemSpec

    spec = ProblemSpec.from_factorized(cc, recipe)
    out = spec.as_dict()
    out["product_factor_count"] = np.int64(int(np.max(spec.product_factors)) + 1)
    np.savez_compressed(path, **out)
    return out


def export_golden(name, fx, cc, path: Path) -> None:
    from c3l.cc.component_tensor import (
        ComponentEOMProblem, ComponentStaticProblem, component_eom_context,
        component_eom_sigma, component_eom_sources, component_static_jvp,
        component_static_residual,
    )
    from c3l.cc.component_response import ComponentSigmaOperator, component_retarded_green
    from c3l.cc.component_solver import solve_component_ccsd
    from c3l.cc.eom import eom_ccsd_problem

    g: dict = {}
    t0 = time.perf_counter()
    static = ComponentStaticProblem.compile(cc, fuse_products=True)
    g["setup_seconds"] = time.perf_counter() - t0
    n = cc.model.n_sites
    idx = np.arange(cc.num_variables, dtype=np.float64)
    T = cc.tilde.unpack(fx["scale"] * np.cos(idx + 0.13))
    D = cc.tilde.unpack(0.2 * np.sin(idx + 0.31))
    g["amplitude_scale"] = np.float64(fx["scale"])
    g["fixed_variables"] = fx["scale"] * np.cos(idx + 0.13)
    g["fixed_direction_variables"] = 0.2 * np.sin(idx + 0.31)
    g["fixed_amplitudes"] = T
    g["fixed_direction"] = D
    t0 = time.perf_counter()
    res = component_static_residual(static, T)
    g["residual_seconds"] = time.perf_counter() - t0
    g["residual"] = res.retained
    g["residual_reference"] = np.complex128(res.reference)
    t0 = time.perf_counter()
    jvp = component_static_jvp(static, T, D)
    g["jvp_seconds"] = time.perf_counter() - t0
    g["jvp"] = jvp.retained
    g["jvp_reference"] = np.complex128(jvp.reference)
    if 4 * n <= 62:
        g["cluster_masks"] = np.asarray(cc.cluster_basis.masks, np.int64)
    g["tilde_partner"] = np.asarray(cc.tilde.partner, np.int64)
    g["tilde_phase"] = np.asarray(cc.tilde.phase, complex)
    g["tilde_independent"] = np.asarray(cc.tilde.independent, np.int64)
    print(f"  [{name}] residual {g['residual_seconds']:.2f}s jvp {g['jvp_seconds']:.2f}s", flush=True)
    if not fx["solve"]:
        if fx.get("eom"):
            _export_eom(g, cc, static, T, fx, name, None)
        np.savez_compressed(path, **g)
        return
    t0 = time.perf_counter()
    sol = solve_component_ccsd(static)
    g["solve_seconds"] = time.perf_counter() - t0
    g["solution_amplitudes"] = sol.amplitudes
    g["solution_variables"] = sol.variables
    g["solution_packed_residual_norm"] = sol.packed_residual_norm
    g["solution_iterations"] = sol.iterations
    g["solution_residual_evaluations"] = sol.residual_evaluations
    g["solution_jvp_evaluations"] = sol.jvp_evaluations
    g["solution_converged"] = sol.converged
    print(f"  [{name}] solve {g['solve_seconds']:.2f}s iters {sol.iterations} |r| {sol.packed_residual_norm:.2e}", flush=True)
    _export_eom(g, cc, static, sol.amplitudes, fx, name, None)
    np.savez_compressed(path, **g)


def _export_eom(g, cc, static, amplitudes, fx, name, _unused) -> None:
    from c3l.cc.component_tensor import (
        ComponentEOMProblem, component_eom_context, component_eom_sigma, component_eom_sources,
    )
    from c3l.cc.component_response import ComponentSigmaOperator, component_retarded_green
    from c3l.cc.eom import eom_ccsd_problem

    n = cc.model.n_sites
    g["eom_amplitudes"] = amplitudes
    eom = eom_ccsd_problem(cc, response_spin=0)
    if 4 * n <= 62:
        g["eom_masks"] = np.asarray(eom.basis.masks, np.int64)
        g["eom_charges"] = np.asarray(eom.basis.charge_labels, np.int64)
    for charge in (1, -1):
        tag = "p" if charge == 1 else "m"
        problem = ComponentEOMProblem.compile(eom, static, charge=charge)
        t0 = time.perf_counter()
        context = component_eom_context(problem, amplitudes)
        g[f"eom{tag}_context_seconds"] = time.perf_counter() - t0
        op = ComponentSigmaOperator(context)
        g[f"eom{tag}_positions"] = np.asarray(problem.positions, np.int64)
        g[f"eom{tag}_diagonal"] = op.diagonal
        dim = op.dimension
        k = np.arange(dim, dtype=np.float64)
        x = np.cos(0.7 * k + 0.2) + 1j * np.sin(0.3 * k - 0.1)
        g[f"eom{tag}_probe"] = x
        t0 = time.perf_counter()
        g[f"eom{tag}_sigma"] = component_eom_sigma(context, x).retained
        g[f"eom{tag}_sigma_seconds"] = time.perf_counter() - t0
        src = component_eom_sources(context)
        g[f"eom{tag}_addition"] = src.addition
        g[f"eom{tag}_removal"] = src.removal
        g[f"eom{tag}_sink"] = src.sink
        if fx["omega"] is not None and charge == 1:
            t0 = time.perf_counter()
            green = component_retarded_green(op, src, fx["omega"], fx["eta"])
            g["green_seconds"] = time.perf_counter() - t0
            g["green_omega"] = green.omega
            g["green_eta"] = np.float64(fx["eta"])
            g["green_addition"] = green.addition
            g["green_removal"] = green.removal
            g["green_retarded"] = green.retarded
            g["green_sigma_calls"] = op.action_calls
            print(f"  [{name}] green {g['green_seconds']:.2f}s ({op.action_calls} sigma calls)", flush=True)


def export_warmstart_family(count: int, path: Path) -> None:
    """Seeded SIAM models (10 pseudomodes, U uniform in [2, 6]) for the learned warm start.

    Only the problem specs are exported: the training targets are the
    amplitudes the GPU solver itself produces on these models.
    """
    from c3l import FermionicLindbladModel
    from c3l.cc.factorized import factorized_cc_problem

    out = {"count": np.int64(count)}
    for i in range(count):
        rng = np.random.default_rng(1000 + i)
        U = float(rng.uniform(2.0, 6.0))
        nm = 10
        eb = rng.uniform(-3, 3, nm)
        V = rng.normal(0, 0.3, nm)
        r = rng.uniform(0.05, 0.5, nm)
        f = 1.0 / (np.exp(eb / 0.1) + 1.0)
        E = np.diag(np.r_[-U / 2, eb]).astype(complex)
        E[0, 1:] = V
        E[1:, 0] = V
        model = FermionicLindbladModel(E, np.diag(np.r_[0, r * (1 - f)]), np.diag(np.r_[0, r * f]), U=U)
        cc = factorized_cc_problem(model, "CCSD", m_up=0.5, reference_mode="legacy_half_filled")
        tmp = HERE / "_tmp_ws.npz"
        spec = export_spec(cc, tmp, "legacy_half_filled:0.5")
        tmp.unlink()
        for k, v in spec.items():
            out[f"m{i}_{k}"] = v
        out[f"m{i}_U"] = np.float64(U)
        print(f"  warm-start model {i}: U={U:.3f}", flush=True)
    np.savez_compressed(path, **out)


COMPACT_SAMPLES = 4096


def compact_golden(path: Path) -> None:
    """Shrink a large golden: drop the deterministic inputs (they are
    regenerated from their formulas), keep reference outputs at a seeded
    sample of coordinates plus their full norms."""
    g = dict(np.load(path))
    out = {}
    rng = np.random.default_rng(12345)
    dim = g["residual"].size
    pos = np.sort(rng.choice(dim, size=min(COMPACT_SAMPLES, dim), replace=False))
    out["compact"] = np.int64(1)
    out["sample_positions"] = pos
    out["scale"] = g["amplitude_scale"]
    for key in ("residual", "jvp"):
        out[f"{key}_sample"] = g[key][pos]
        out[f"{key}_norm"] = np.float64(np.linalg.norm(g[key]))
    for key in ("residual_reference", "jvp_reference", "setup_seconds", "residual_seconds", "jvp_seconds"):
        if key in g:
            out[key] = g[key]
    for tag in ("p", "m"):
        if f"eom{tag}_sigma" not in g:
            continue
        d = g[f"eom{tag}_sigma"].size
        ep = np.sort(rng.choice(d, size=min(COMPACT_SAMPLES, d), replace=False))
        out[f"eom{tag}_sample_positions"] = ep
        out[f"eom{tag}_dimension"] = np.int64(d)
        out[f"eom{tag}_sigma_sample"] = g[f"eom{tag}_sigma"][ep]
        out[f"eom{tag}_sigma_norm"] = np.float64(np.linalg.norm(g[f"eom{tag}_sigma"]))
        for key in ("addition", "removal", "sink", "diagonal"):
            out[f"eom{tag}_{key}_sample"] = g[f"eom{tag}_{key}"][ep]
        for key in ("context_seconds", "sigma_seconds"):
            if f"eom{tag}_{key}" in g:
                out[f"eom{tag}_{key}"] = g[f"eom{tag}_{key}"]
    np.savez_compressed(path, **out)


MATRIX_GREEN = {
    # n = 9 Kanamori: charge +1
    "kanamori3x2": dict(sites=(0, 1, 2), omega=np.linspace(-6.0, 6.0, 61), eta=0.2, maximum_krylov_dimension=1062,
                        charges=(1,)),
    # n = 27 Kanamori (the three-orbital, eight-mode workload's model): charge +1 and -1,
    # eta = 0.02 on a short grid of [-10, 10]
    "kanamori3x8": dict(sites=(0, 1, 2), omega=np.linspace(-10.0, 10.0, 41), eta=0.02, maximum_krylov_dimension=1600,
                        charges=(1, -1)),
}


def export_matrix_green(fixture: str) -> None:
    """Matrix G^R_ab(omega) of the reference's one-sided Arnoldi driver
    (component_retarded_matrix_green_arnoldi) for the three impurity orbitals
    of a Kanamori fixture at the fixture's fixed amplitudes, written to
    ``<fixture>.matrix.npz`` (charge +1) and ``<fixture>.matrix_m.npz`` (charge -1)."""
    from c3l.cc.component_response import ComponentSigmaOperator, component_retarded_matrix_green_arnoldi
    from c3l.cc.component_tensor import (
        ComponentEOMProblem, ComponentStaticProblem, component_eom_context, component_eom_sources,
    )
    from c3l.cc.eom import eom_ccsd_problem

    spec = MATRIX_GREEN[fixture]
    fx = FIXTURES[fixture]
    cc = build_problem(fx)
    static = ComponentStaticProblem.compile(cc)
    golden = np.load(HERE / f"{fixture}.golden.npz")
    if "eom_amplitudes" in golden.files:
        amplitudes = golden["eom_amplitudes"]
    else:  # compact golden: the fixed amplitudes from their formula
        idx = np.arange(cc.num_variables, dtype=np.float64)
        amplitudes = cc.tilde.unpack(fx["scale"] * np.cos(idx + 0.13))
    for charge in spec["charges"]:
        _export_matrix_charge(fixture, spec, cc, static, amplitudes, charge)


def _export_matrix_charge(fixture, spec, cc, static, amplitudes, charge) -> None:
    from c3l.cc.component_response import ComponentSigmaOperator, component_retarded_matrix_green_arnoldi
    from c3l.cc.component_tensor import ComponentEOMProblem, component_eom_context, component_eom_sources
    from c3l.cc.eom import eom_ccsd_problem

    path = HERE / (f"{fixture}.matrix.npz" if charge == 1 else f"{fixture}.matrix_m.npz")
    problem = ComponentEOMProblem.compile(eom_ccsd_problem(cc, response_spin=0), static, charge=charge)
    context = component_eom_context(problem, amplitudes)
    op = ComponentSigmaOperator(context)
    sources = [component_eom_sources(context, site=s) for s in spec["sites"]]
    t0 = time.perf_counter()
    res = component_retarded_matrix_green_arnoldi(op, sources, spec["omega"], spec["eta"],
                                                  maximum_krylov_dimension=spec["maximum_krylov_dimension"])
    seconds = time.perf_counter() - t0
    np.savez_compressed(
        path, charge=np.int64(charge), omega=res.omega, eta=np.float64(res.eta), sites=np.asarray(res.sites, np.int64),
        addition=res.addition, removal=res.removal, retarded=res.retarded,
        addition_relative_residuals=res.addition_relative_residuals,
        removal_relative_residuals=res.removal_relative_residuals,
        addition_dimensions=np.asarray([p.dimension for p in res.addition_projections], np.int64),
        removal_dimensions=np.asarray([p.dimension for p in res.removal_projections], np.int64),
        maximum_krylov_dimension=np.int64(spec["maximum_krylov_dimension"]), seconds=np.float64(seconds),
        action_calls=np.int64(res.component_action_calls))
    print(f"  matrix green {seconds:.1f}s, dims {[p.dimension for p in res.addition_projections]} "
          f"{[p.dimension for p in res.removal_projections]}", flush=True)


DRIVERS = {
    # fixture: source sites, GMRES matrix frequencies/eta, shifts (Matsubara points
    # i(2k+1)pi/beta and real-axis points omega + i eta), time grid, time validation shifts
    "twosrc": dict(sites=(0, 1), gmres_omega=np.linspace(-2.0, 2.0, 9), gmres_eta=0.1,
                   shifts=np.r_[1j * (2 * np.arange(6) + 1) * np.pi / 8.0, np.linspace(-2.0, 2.0, 5) + 0.1j],
                   time=np.linspace(0.0, 12.0, 49), validation=np.linspace(-2.0, 2.0, 5) + 0.1j, beta=8.0, n_iw=6),
    "siam10": dict(sites=(0,), gmres_omega=np.asarray([-1.0, 0.0, 1.5]), gmres_eta=0.2,
                   shifts=np.r_[1j * (2 * np.arange(6) + 1) * np.pi / 10.0, np.linspace(-8.0, 8.0, 41) + 0.5j],
                   time=np.linspace(0.0, 20.0, 81), validation=np.linspace(-4.0, 4.0, 9) + 0.2j, beta=10.0, n_iw=16),
}


# the reference's full S1 + S3 + S5 response action (its rank-five shell) at the
# fixture's fixed amplitudes: one action per (response spin, charge), G^R on a
# short grid for the two smallest models
S135 = {
    "readme": dict(green=True, omega=np.linspace(-4.0, 4.0, 9), eta=0.1),
    "s135fix": dict(green=True, omega=np.linspace(-3.0, 3.0, 7), eta=0.05),
    "twosrc": dict(green=False),
    "kanamori3x2": dict(green=False),
}


S135_FULL_MAX = 5000  # larger S135 actions keep sampled outputs only


def s135_seed(spin: int, charge: int) -> int:
    return 20260722 + 2 * spin + (charge > 0)


def s135_sample(tag: str, y, p_dimension: int, diagonal, s5_keys, s5_tuples) -> dict:
    """Every S13 coordinate and 4,000 seeded rank-five coordinates of an action:
    the outputs, the diagonal and the shell's keys and index tuples there."""
    rng = np.random.default_rng(7)
    idx = np.concatenate([np.arange(p_dimension),
                          np.sort(rng.choice(np.arange(p_dimension, y.size), 4000, replace=False))])
    s5 = idx[idx >= p_dimension] - p_dimension
    return {f"{tag}_y_index": idx.astype(np.int64), f"{tag}_y_sample": y[idx], f"{tag}_dimension": np.int64(y.size),
            f"{tag}_diagonal_sample": diagonal[idx], f"{tag}_s5_index": s5.astype(np.int64),
            f"{tag}_s5_keys_sample": s5_keys[s5].astype(np.int8), f"{tag}_s5_tuples_sample": s5_tuples[s5].astype(np.int8),
            f"{tag}_s5_dimension": np.int64(s5_keys.shape[0])}


def export_s135(name: str, path: Path) -> None:
    """``CompiledFullS135Action`` / ``FullS135ResponseOperator``
    (``src/c3l/cc/s135_full.py:101``, ``:296``): the action on a seeded vector,
    the rapidity diagonal and the S5 coordinate order (block keys and index
    tuples) for response spins 0 and 1 and charges +1 and -1; G^R of site 0
    through the S135 operator (``component_retarded_green`` pads the S13
    sources with zeros) where cheap."""
    from c3l.cc.component_response import component_retarded_matrix_green_arnoldi
    from c3l.cc.component_tensor import (
        ComponentEOMProblem, ComponentStaticProblem, component_eom_context, component_eom_sources,
    )
    from c3l.cc.eom import eom_ccsd_problem
    from c3l.cc.s135_full import CompiledFullS135Action, FullS135ResponseOperator, rapidity_diagonal

    spec = S135[name]
    cc = build_problem(FIXTURES[name])
    static = ComponentStaticProblem.compile(cc)
    golden = np.load(HERE / f"{name}.golden.npz")
    amplitudes = golden["eom_amplitudes" if "eom_amplitudes" in golden.files else "solution_amplitudes"]
    out: dict = {}
    for spin in (0, 1):
        eom = eom_ccsd_problem(cc, response_spin=spin, build_next_rank_masks=False)
        for charge in (1, -1):
            t0 = time.perf_counter()
            problem = ComponentEOMProblem.compile(eom, static, charge)
            context = component_eom_context(problem, amplitudes)
            op = FullS135ResponseOperator(CompiledFullS135Action(context))
            tag = f"s{spin}q{'p' if charge == 1 else 'm'}"
            rng = np.random.default_rng(s135_seed(spin, charge))
            x = rng.normal(size=op.dimension) + 1j * rng.normal(size=op.dimension)
            y = op.matvec(x)
            diagonal = rapidity_diagonal(cc.rapidities, op.coordinates)
            keys, tuples = [], []
            for blk in op.S5.blocks:
                keys.append(np.broadcast_to(np.asarray(blk.key, np.int64), (blk.vector_positions.size, 4)))
                tuples.append(np.pad(blk.indices, ((0, 0), (0, 5 - blk.indices.shape[1])), constant_values=-1))
                assert np.array_equal(blk.vector_positions, np.arange(blk.vector_positions[0],
                                                                      blk.vector_positions[0] + blk.vector_positions.size))
            keys, tuples = np.concatenate(keys), np.concatenate(tuples)
            out[f"{tag}_p_dimension"] = np.int64(op.p_dimension)
            if op.dimension <= S135_FULL_MAX:
                out.update({f"{tag}_x": x, f"{tag}_y": y, f"{tag}_diagonal": diagonal, f"{tag}_s5_keys": keys,
                            f"{tag}_s5_tuples": tuples})
            else:  # the input is regenerated from its seed; the rest kept at sampled coordinates
                out.update(s135_sample(tag, y, op.p_dimension, diagonal, keys, tuples))
            if spec["green"] and spin == 0:
                # the reference's S135 G^R goes through its Arnoldi drivers (the S135
                # operator has no Jacobi diagonal for the per-frequency GMRES)
                src = component_eom_sources(context, site=0)

                class Counted:  # the call counters the reference's matrix driver reads
                    dimension = op.dimension
                    action_calls = 0
                    action_wall_seconds = 0.0

                    def matvec(self, v):
                        self.action_calls += 1
                        return op.matvec(v)

                res = component_retarded_matrix_green_arnoldi(Counted(), [src], spec["omega"], spec["eta"])
                out[f"{tag}_green_omega"] = np.asarray(spec["omega"])
                out[f"{tag}_green_eta"] = np.float64(spec["eta"])
                out[f"{tag}_green_retarded"] = np.asarray(res.retarded)[:, 0, 0]
                out[f"{tag}_green_addition"] = np.asarray(res.addition)[:, 0, 0]
            print(f"[{name}] S135 spin {spin} charge {charge:+d}: dim {op.dimension} "
                  f"(S13 {op.p_dimension}) {time.perf_counter() - t0:.1f}s", flush=True)
    np.savez_compressed(path, **out)


def export_spectra(path: Path) -> None:
    """The reference's spectra reconstruction (``src/c3l/spectra/reconstruction.py``)
    on the siam10 CCSD G^R (its full 1,001-omega golden) and on the n = 9
    Kanamori model's 3 x 3 impurity block: the auxiliary G0, the scalar
    auxiliary self-energy and physical Dyson reconstruction (G^K from the
    equilibrium relation at T = 0.1; a semicircular target bath), the matrix
    self-energy, Dyson and ordered reconstruction, and the diagnostics."""
    from c3l.matsubara.dyson import noninteracting_retarded_green
    from c3l.spectra import reconstruction as rc

    out: dict = {}
    g = np.load(HERE / "siam10.golden.npz")
    model = FIXTURES["siam10"]["model"]()
    w = np.asarray(g["green_omega"], np.float64)
    gr = np.asarray(g["green_retarded"])
    g0r, g0k = rc.noninteracting_auxiliary_green(model, w, eta=0.05)
    gk = (gr - gr.conj()) * np.tanh(w / 0.2)
    sr, sk = rc.auxiliary_self_energy(g0r, g0k, gr, gk)
    z = w + 0.05j
    dr = 0.09 * (z - np.sqrt(z - 2.0 + 0j) * np.sqrt(z + 2.0 + 0j)) / 2.0
    dk = (dr - dr.conj()) * np.tanh(w / 0.2)
    phys = rc.physical_dyson_reconstruction(w, -2.0, dr, dk, sr, sk)
    out.update(scalar_omega=w, scalar_G_R=gr, scalar_G_K=gk, scalar_G0_R=g0r, scalar_G0_K=g0k, scalar_Sigma_R=sr,
               scalar_Sigma_K=sk, scalar_Delta_R=dr, scalar_Delta_K=dk, phys_retarded=phys.retarded,
               phys_keldysh=phys.keldysh, phys_spectral=phys.spectral,
               fdt_defect=np.float64(rc.equilibrium_fdt_defect(w, gr, gk, 0.1)),
               ph_defect=np.float64(rc.particle_hole_spectral_defect(w, -gr.imag / np.pi)),
               grid_diagnostics=np.asarray(list(rc.spectral_grid_diagnostics(w, gr).values())))
    # matrix forms on the Kanamori impurity block (3 orbitals), real axis with broadening
    kmodel = FIXTURES["kanamori3x2"]["model"]()
    wm = np.linspace(-3.0, 3.0, 61)
    zm = wm + 0.1j
    G0 = noninteracting_retarded_green(kmodel, zm, (0, 1, 2))
    rng = np.random.default_rng(11)
    S = rng.normal(size=(3, 3)) + 1j * rng.normal(size=(3, 3))
    sigma = 0.1 * (S + S.conj().T) / 2 - 0.05j * np.eye(3)
    G = np.linalg.inv(np.linalg.inv(G0) - sigma[None])
    mse = rc.matrix_auxiliary_self_energy(G0, G)
    h = np.asarray(kmodel.E)[np.ix_((0, 1, 2), (0, 1, 2))]
    delta_pm = zm[:, None, None] * np.eye(3)[None] - h[None] - np.linalg.inv(G0)
    delta_ph = 0.09 * ((zm - np.sqrt(zm - 2.0 + 0j) * np.sqrt(zm + 2.0 + 0j)) / 2.0)[:, None, None] * np.eye(3)[None]
    md = rc.matrix_dyson_green(zm, h, delta_ph, mse.retarded)
    mo = rc.matrix_ordered_dyson_reconstruction(G, delta_pm, delta_ph)
    out.update(matrix_z=zm, matrix_G0=G0, matrix_G=G, matrix_h=h, matrix_Delta_PM=delta_pm, matrix_Delta_phys=delta_ph,
               mse_retarded=mse.retarded, mse_G0_cond=mse.G0_condition_number, mse_G_cond=mse.G_condition_number,
               mse_dyson_right=mse.dyson.right_backward_residual, mse_dyson_left=mse.dyson.left_backward_residual,
               md_retarded=md.retarded, md_inverse=md.inverse_retarded, md_cond=md.resolvent.condition_number,
               md_right=md.resolvent.right_backward_residual, md_left=md.resolvent.left_backward_residual,
               md_spectral=md.spectral.spectral, md_min_eig=md.spectral.minimum_eigenvalue,
               md_max_eig=md.spectral.maximum_eigenvalue, md_neg=md.spectral.negative_ratio,
               md_herm=md.spectral.hermiticity_defect,
               mo_retarded=mo.retarded, mo_right_order=mo.retarded_from_right_order,
               mo_left_res=mo.left_ordered_residual, mo_right_res=mo.right_ordered_residual,
               mo_left_id=mo.left_resolvent_identity_residual, mo_right_id=mo.right_resolvent_identity_residual,
               mo_diff=mo.ordering_difference, mo_left_cond=mo.left_operator_condition_number,
               mo_right_cond=mo.right_operator_condition_number)
    np.savez_compressed(path, **out)


# the reference's solve_matsubara on fixed amplitudes (the converged siam10
# root; the fixed Kanamori amplitudes of the EOM goldens), both spin blocks
MATSUBARA = {
    "siam10": dict(beta=10.0, n_iw=8),
    "kanamori3x2": dict(beta=8.0, n_iw=6),
    "readme": dict(beta=10.0, n_iw=6, ranks=("S13", "S135")),
}


def export_matsubara(name: str, path: Path) -> None:
    """``solve_matsubara`` (``src/c3l/matsubara/solver.py:100``) with the
    fixture's amplitudes (the static solve skipped), the default impurity block
    (the interaction sites) and response spins 0 and 1 (and, where the table
    asks, the S135 response space); plus the Dyson re-insertion into a
    semicircular target bath (half-bandwidth 2, hopping 0.3)."""
    from c3l.cc.component_tensor import ComponentStaticProblem
    from c3l.matsubara.grid import matsubara_grid
    from c3l.matsubara.solver import solve_matsubara

    spec = MATSUBARA[name]
    cc = build_problem(FIXTURES[name])
    static = ComponentStaticProblem.compile(cc)
    golden = np.load(HERE / f"{name}.golden.npz")
    amplitudes = golden["eom_amplitudes" if "eom_amplitudes" in golden.files else "solution_amplitudes"]
    grid = matsubara_grid(spec["beta"], n_iw=spec["n_iw"])
    # the amplitudes are the fixture golden's (not stored again)
    out: dict = {"beta": np.float64(spec["beta"]), "indices": np.asarray(grid.indices, np.int64)}
    z = grid.iw
    target = (0.09 * (z - np.sign(z.imag) * np.sqrt(z ** 2 - 4.0 + 0j)) / 2.0)
    for rank in spec.get("ranks", ("S13",)):
        for spin in (0, 1):
            t0 = time.perf_counter()
            sol = solve_matsubara(static, grid, amplitudes=amplitudes, response_spin=spin, rank=rank)
            m = len(sol.sites)
            hyb = np.broadcast_to(target[:, None, None] * np.eye(m), (len(grid), m, m))
            tag = f"s{spin}" if rank == "S13" else f"s{spin}_{rank}"
            out.update({f"{tag}_green": sol.green, f"{tag}_self_energy": sol.self_energy,
                        f"{tag}_noninteracting": sol.noninteracting, f"{tag}_hybridization": sol.hybridization,
                        f"{tag}_dyson_target": sol.dyson(hyb), f"{tag}_seconds": np.float64(time.perf_counter() - t0)})
            out["sites"] = np.asarray(sol.sites, np.int64)
            out["one_body"] = sol.one_body
            out["static_residual"] = np.float64(sol.static_residual)
            print(f"[{name}] matsubara {rank} spin {spin}: sites {sol.sites} {time.perf_counter() - t0:.1f}s",
                  flush=True)
    out["dyson_target_hybridization"] = target
    np.savez_compressed(path, **out)


def export_drivers(name: str, path: Path) -> None:
    """The reference's other response drivers on a fixture's converged
    amplitudes, charge +1: component_retarded_matrix_green (one GMRES solve per
    source, channel and frequency), component_retarded_matrix_green_shifts
    (complex shifts), component_retarded_time (first site) and
    component_retarded_matrix_time (with the separate channels), and
    component_matsubara_green on a symmetric explicit Matsubara grid."""
    from c3l.cc.component_response import (
        ComponentSigmaOperator, component_retarded_matrix_green, component_retarded_matrix_green_shifts,
        component_retarded_matrix_time, component_retarded_time,
    )
    from c3l.cc.component_tensor import (
        ComponentEOMProblem, ComponentStaticProblem, component_eom_context, component_eom_sources,
    )
    from c3l.cc.eom import eom_ccsd_problem

    spec = DRIVERS[name]
    cc = build_problem(FIXTURES[name])
    static = ComponentStaticProblem.compile(cc)
    golden = np.load(HERE / f"{name}.golden.npz")
    amplitudes = golden["eom_amplitudes" if "eom_amplitudes" in golden.files else "solution_amplitudes"]
    problem = ComponentEOMProblem.compile(eom_ccsd_problem(cc, response_spin=0), static, charge=1)
    context = component_eom_context(problem, amplitudes)
    sources = [component_eom_sources(context, site=s) for s in spec["sites"]]
    out: dict = {"sites": np.asarray(spec["sites"], np.int64)}
    t0 = time.perf_counter()
    op = ComponentSigmaOperator(context)
    mg = component_retarded_matrix_green(op, sources, spec["gmres_omega"], spec["gmres_eta"])
    out.update(gmres_omega=mg.omega, gmres_eta=np.float64(mg.eta), gmres_addition=mg.addition,
               gmres_removal=mg.removal, gmres_retarded=mg.retarded, gmres_calls=np.int64(op.action_calls),
               gmres_seconds=np.float64(time.perf_counter() - t0))
    t0 = time.perf_counter()
    op = ComponentSigmaOperator(context)
    sh = component_retarded_matrix_green_shifts(op, sources, spec["shifts"])
    out.update(shifts=sh.shifts, shifts_addition=sh.addition, shifts_removal=sh.removal,
               shifts_retarded=sh.retarded, shifts_addition_relative_residuals=sh.addition_relative_residuals,
               shifts_removal_relative_residuals=sh.removal_relative_residuals,
               shifts_addition_dimensions=np.asarray([p.dimension for p in sh.addition_projections], np.int64),
               shifts_removal_dimensions=np.asarray([p.dimension for p in sh.removal_projections], np.int64),
               shifts_action_calls=np.int64(sh.action_calls), shifts_seconds=np.float64(time.perf_counter() - t0))
    t0 = time.perf_counter()
    op = ComponentSigmaOperator(context)
    out["time"] = spec["time"]
    out["time_retarded"] = component_retarded_time(op, sources[0], spec["time"])
    out["time_calls"] = np.int64(op.action_calls)
    out["time_seconds"] = np.float64(time.perf_counter() - t0)
    t0 = time.perf_counter()
    op = ComponentSigmaOperator(context)
    mt = component_retarded_matrix_time(op, sources, spec["time"], spec["validation"])
    out.update(validation_shifts=spec["validation"], mtime_retarded=mt.retarded, mtime_addition=mt.addition,
               mtime_removal=mt.removal, mtime_channel_sum_defect=np.float64(mt.channel_sum_defect),
               mtime_combined_relative_time_residuals=mt.combined_relative_time_residuals,
               mtime_addition_relative_time_residuals=mt.addition_relative_time_residuals,
               mtime_removal_relative_time_residuals=mt.removal_relative_time_residuals,
               mtime_combined_dimensions=np.asarray([p.dimension for p in mt.combined_projections], np.int64),
               mtime_calls=np.int64(op.action_calls), mtime_seconds=np.float64(time.perf_counter() - t0))
    from c3l.matsubara.grid import matsubara_grid
    from c3l.matsubara.solver import component_matsubara_green

    grid = matsubara_grid(spec["beta"], n_iw=spec["n_iw"])
    op = ComponentSigmaOperator(context)
    mats = component_matsubara_green(op, sources, grid)
    out.update(matsubara_beta=np.float64(grid.beta), matsubara_indices=grid.indices, matsubara_green=mats.green,
               matsubara_max_relative_residual=np.float64(mats.max_relative_residual))
    np.savez_compressed(path, **out)
    print(f"  [{name}] drivers: gmres {out['gmres_seconds']:.1f}s shifts {out['shifts_seconds']:.1f}s "
          f"time {out['time_seconds']:.1f}s matrix time {out['mtime_seconds']:.1f}s", flush=True)


ED_CHECK = dict(fixture="readme", omega=np.linspace(-4.0, 4.0, 161), eta=0.1)


def export_ed(path: Path) -> None:
    """Exact Lindblad-ED G^R of the README model and the reference's CCSD-EOM
    (S1 + S3) G^R on the same grid: the exact-diagonalisation check of the
    reference's examples/basic/01_ccsd_eom.py (ED by its examples/siam_ed
    sector code, no dense Liouvillian), run here once by the reference."""
    from c3l.cc.component_response import ComponentSigmaOperator, component_retarded_green
    from c3l.cc.component_solver import solve_component_ccsd
    from c3l.cc.component_tensor import (
        ComponentEOMProblem, ComponentStaticProblem, component_eom_context, component_eom_sources,
    )
    from c3l.cc.eom import eom_ccsd_problem

    sys.path.insert(0, str(Path(sys.modules["c3l"].__file__).resolve().parents[2] / "examples"))
    from siam_ed.physical_sparse import (
        compile_physical_sector_operator, physical_density_action, physical_response_action,
        physical_response_vectors, solve_trace_fixed_static,
    )
    from siam_ed.sparse_response import sparse_direct_resolvent

    fx = FIXTURES[ED_CHECK["fixture"]]
    omega, eta = ED_CHECK["omega"], ED_CHECK["eta"]
    cc = build_problem(fx)
    model = cc.model
    static = ComponentStaticProblem.compile(cc)
    sol = solve_component_ccsd(static)
    problem = ComponentEOMProblem.compile(eom_ccsd_problem(cc, response_spin=0), static, charge=1)
    context = component_eom_context(problem, sol.amplitudes)
    op = ComponentSigmaOperator(context)
    green = component_retarded_green(op, component_eom_sources(context), omega, eta)
    density = compile_physical_sector_operator(physical_density_action(model), maximum_bytes=1 << 30)
    ness = solve_trace_fixed_static(density)
    response = compile_physical_sector_operator(physical_response_action(model, spin=0, charge=1),
                                                maximum_bytes=1 << 30)
    vectors = physical_response_vectors(density.action.sector, ness.coefficients,
                                        model.orbital_index(model.impurity_site, 0))
    sources = np.column_stack((vectors.creation_left, vectors.creation_right))
    ed = sparse_direct_resolvent(response, sources, omega.astype(np.complex128) + 1j * eta,
                                 verification_operator=response.action)
    channels = ed.transfer(vectors.annihilation_sink)[:, 0, :]
    g_ed = channels[:, 0] + channels[:, 1]
    dev = float(np.max(np.abs(green.retarded - g_ed)) / np.max(np.abs(g_ed)))
    np.savez_compressed(path, omega=omega, eta=np.float64(eta), green_ed=g_ed, green_cc_reference=green.retarded,
                        cc_vs_ed_relative=np.float64(dev))
    print(f"  ED check: CCSD-EOM vs ED max relative deviation {dev:.3e}", flush=True)


def main() -> None:
    parser = argparse.ArgumentParser()
    parser.add_argument("--reference", default=str(HERE.parents[2] / "reference" / "src"))
    parser.add_argument("names", nargs="*")
    args = parser.parse_args()
    _import_reference(args.reference)
    if args.names == ["warmstart"]:
        export_warmstart_family(64, HERE / "warmstart_siam.npz")
        return
    if args.names and args.names[0] == "matrix":
        for fixture in args.names[1:] or ["kanamori3x2"]:
            export_matrix_green(fixture)
        return
    if args.names == ["ed"]:
        export_ed(HERE / f"{ED_CHECK['fixture']}.ed.npz")
        return
    if args.names and args.names[0] == "spec":
        for name in args.names[1:] or list(SPEC_ONLY):
            t0 = time.perf_counter()
            model, reference = build_reference(SPEC_ONLY[name])
            cc = light_problem(model, reference)
            export_spec(cc, HERE / f"{name}.spec.npz", SPEC_ONLY[name]["recipe"])
            print(f"[{name}] n={model.n_sites} products={len(cc.products)} spec {time.perf_counter() - t0:.1f}s",
                  flush=True)
        return
    if args.names and args.names[0] == "model":
        # add the physical one-body model to committed specs without rebuilding them
        sys.path.insert(0, str(HERE.parents[1]))
        from c3lindblad_gb300.spec import model_fields

        for name in args.names[1:] or [*FIXTURES, *SPEC_ONLY]:
            fx = FIXTURES.get(name) or SPEC_ONLY[name]
            path = HERE / f"{name}.spec.npz"
            data = dict(np.load(path))
            data.update(model_fields(fx["model"]()))
            np.savez_compressed(path, **data)
            print(f"[{name}] model added", flush=True)
        return
    if args.names and args.names[0] == "static":
        # the static goldens only (fixed-amplitude residual and JVP, tilde map),
        # for fixtures whose EOM goldens take the reference hours
        for name in args.names[1:]:
            fx = dict(FIXTURES[name], solve=False, eom=False)
            cc = build_problem(fx)
            export_golden(name, fx, cc, HERE / f"{name}.golden.npz")
        return
    if args.names == ["spectra"]:
        export_spectra(HERE / "spectra.reconstruction.npz")
        return
    if args.names and args.names[0] == "s135":
        for name in args.names[1:] or list(S135):
            export_s135(name, HERE / f"{name}.s135.npz")
        return
    if args.names and args.names[0] == "matsubara":
        for name in args.names[1:] or list(MATSUBARA):
            export_matsubara(name, HERE / f"{name}.matsubara.npz")
        return
    if args.names and args.names[0] == "drivers":
        for name in args.names[1:] or list(DRIVERS):
            export_drivers(name, HERE / f"{name}.drivers.npz")
        return
    names = args.names or list(FIXTURES)
    for name in names:
        fx = FIXTURES[name]
        t0 = time.perf_counter()
        cc = build_problem(fx)
        print(f"[{name}] n={cc.model.n_sites} amps={cc.num_amplitudes} products={len(cc.products)} "
              f"setup {time.perf_counter() - t0:.1f}s", flush=True)
        export_spec(cc, HERE / f"{name}.spec.npz", fx["recipe"])
        export_golden(name, fx, cc, HERE / f"{name}.golden.npz")
        if cc.model.n_sites > 16:
            compact_golden(HERE / f"{name}.golden.npz")


if __name__ == "__main__":
    main()
