"""The full S1 + S3 + S5 response action against the reference's own
``FullS135ResponseOperator`` (``src/c3l/cc/s135_full.py:101-361``).

The goldens (``*.s135.npz``, written by ``make_fixtures.py s135``) hold the
reference's action on a seeded vector for response spins 0, 1 and charges
+1, -1 at the fixture's fixed amplitudes, its rapidity diagonal, the order of
its rank-five shell coordinates, and (readme, s135fix) G^R of site 0 through
the S135 operator.  Larger actions keep every S13 output and 4,000 sampled
rank-five outputs; their input is regenerated from its seed.  The CPU tests
run the compiled S135 program through the NumPy plan interpreter; the GPU
tests run the device operator through the C ABI.  The bar is the reference's
own test of this action against its explicit response matrix (3e-11).
"""

from __future__ import annotations

import numpy as np
import pytest

from conftest import GOLDEN, eom_amplitudes, relerr

NAMES = [p.name[: -len(".s135.npz")] for p in sorted(GOLDEN.glob("*.s135.npz"))]
BLOCKS = [(spin, charge) for spin in (0, 1) for charge in (1, -1)]


@pytest.fixture(scope="module")
def plans():
    from c3lindblad_gb300.plans import StaticPlan
    from conftest import load

    cache = {}

    def get(name):
        if name not in cache:
            spec, g = load(name)
            cache[name] = (spec, g, StaticPlan(spec))
        return cache[name]

    return get


def _tag(spin, charge):
    return f"s{spin}q{'p' if charge == 1 else 'm'}"


def _seed(spin, charge):
    return 20260722 + 2 * spin + (charge > 0)


def _case(name, spin, charge):
    """(x, index of the compared outputs, reference outputs there)."""
    ref = np.load(GOLDEN / f"{name}.s135.npz")
    k = _tag(spin, charge)
    if f"{k}_x" in ref.files:
        x = ref[f"{k}_x"]
        return ref, x, np.arange(x.size), ref[f"{k}_y"]
    dim = int(ref[f"{k}_dimension"])
    rng = np.random.default_rng(_seed(spin, charge))
    x = rng.normal(size=dim) + 1j * rng.normal(size=dim)
    return ref, x, ref[f"{k}_y_index"], ref[f"{k}_y_sample"]


@pytest.mark.parametrize("name", NAMES)
@pytest.mark.parametrize("spin,charge", BLOCKS)
def test_coordinates_follow_the_reference_shell(name, spin, charge):
    from c3lindblad_gb300.layout import eom_coordinates
    from c3lindblad_gb300.spec import ProblemSpec

    spec = ProblemSpec.load(GOLDEN / f"{name}.spec.npz")
    ref = np.load(GOLDEN / f"{name}.s135.npz")
    k = _tag(spin, charge)
    c = eom_coordinates(spec.n, spin, charge, "S135")
    p = int(ref[f"{k}_p_dimension"])
    s13 = eom_coordinates(spec.n, spin, charge)
    w = s13.tuples.shape[1]
    assert np.array_equal(c.tuples[:p, :w], s13.tuples) and np.all(c.tuples[:p, w:] == -1)
    if f"{k}_s5_keys" in ref.files:
        sel, keys, tuples = np.arange(ref[f"{k}_s5_keys"].shape[0]), ref[f"{k}_s5_keys"], ref[f"{k}_s5_tuples"]
    else:
        sel, keys, tuples = ref[f"{k}_s5_index"], ref[f"{k}_s5_keys_sample"], ref[f"{k}_s5_tuples_sample"]
    s5 = int(ref[f"{k}_s5_keys"].shape[0]) if f"{k}_s5_keys" in ref.files else int(ref[f"{k}_s5_dimension"])
    assert c.dimension == p + s5
    assert np.array_equal(np.asarray([c.keys[b] for b in c.block_of[p + sel]]), keys)
    assert np.array_equal(c.tuples[p + sel], tuples)


@pytest.mark.parametrize("name", NAMES)
@pytest.mark.parametrize("spin,charge", BLOCKS)
def test_compiled_s135_program_matches_reference(name, spin, charge, plans):
    from c3lindblad_gb300.plans import EOMPlan
    from plan_interpreter import InterpretedEOM

    spec, g, plan = plans(name)
    ref, x, idx, want = _case(name, spin, charge)
    ep = EOMPlan(plan, spin, charge, "S135")
    assert ep.dimension == x.size
    k = _tag(spin, charge)
    if f"{k}_diagonal" in ref.files:
        assert relerr(ep.diagonal, ref[f"{k}_diagonal"]) < 1e-14
    else:
        assert relerr(ep.diagonal[idx], ref[f"{k}_diagonal_sample"]) < 1e-14
    y = InterpretedEOM(ep, eom_amplitudes(g)).sigma(x)
    assert relerr(y[idx], want) < 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("name", NAMES)
def test_device_s135_action_matches_reference(name, cuda_device):
    import c3lindblad_gb300 as c3

    spec = c3.ProblemSpec.load(GOLDEN / f"{name}.spec.npz")
    g = np.load(GOLDEN / f"{name}.golden.npz")
    p = c3.ComponentStaticProblem.compile(spec, device=cuda_device)
    for spin, charge in BLOCKS:
        ref, x, idx, want = _case(name, spin, charge)
        ep = c3.ComponentEOMProblem(p, spin, charge)
        ctx = c3.component_eom_context(ep, eom_amplitudes(g))
        op = c3.FullS135ResponseOperator(c3.CompiledFullS135Action(ctx))
        assert op.dimension == x.size and op.p_dimension == int(ref[f"{_tag(spin, charge)}_p_dimension"])
        assert op.p_dimension + op.s5_dimension == op.dimension
        assert relerr(op.matvec(x)[idx], want) < 3e-11
        with pytest.raises(ValueError, match="full-S135"):
            op.matvec(x[:-1])


@pytest.mark.gpu
@pytest.mark.parametrize("name", [n for n in NAMES if "s0qp_green_retarded" in np.load(GOLDEN / f"{n}.s135.npz").files])
def test_s135_green_matches_reference(name, cuda_device):
    """G^R of site 0 through the S135 operator (the S13 sources padded with
    zeros), by the device Arnoldi resolvent, against the reference's matrix
    Arnoldi driver on its own S135 operator."""
    import c3lindblad_gb300 as c3

    spec = c3.ProblemSpec.load(GOLDEN / f"{name}.spec.npz")
    g = np.load(GOLDEN / f"{name}.golden.npz")
    p = c3.ComponentStaticProblem.compile(spec, device=cuda_device)
    for charge in (1, -1):
        ref = np.load(GOLDEN / f"{name}.s135.npz")
        k = _tag(0, charge)
        ctx = c3.component_eom_context(c3.ComponentEOMProblem(p, 0, charge), eom_amplitudes(g))
        op = c3.FullS135ResponseOperator(c3.CompiledFullS135Action(ctx))
        src = c3.component_eom_sources(ctx, site=0)
        res = c3.component_retarded_green(op, src, ref[f"{k}_green_omega"], float(ref[f"{k}_green_eta"]))
        assert relerr(res.retarded, ref[f"{k}_green_retarded"]) < 1e-8
        assert relerr(res.addition, ref[f"{k}_green_addition"]) < 1e-8
        # the S13 operator gives a different (truncated) answer on the same grid
        s13 = c3.component_retarded_green(c3.ComponentSigmaOperator(ctx), src, ref[f"{k}_green_omega"],
                                          float(ref[f"{k}_green_eta"]))
        assert relerr(s13.retarded, ref[f"{k}_green_retarded"]) > 1e-6
