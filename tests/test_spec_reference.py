"""The drop-in boundary lowers the reference's own objects to the committed specs.

``ComponentStaticProblem.compile(cc)`` accepts the reference's
``FactorizedCCProblem`` / ``ComponentStaticProblem`` and lowers it with
``ProblemSpec.from_reference`` (``src/c3l/cc/component_tensor.py:1276``,
``src/c3l/cc/factorized.py:445``).  These tests build each small fixture model
with the reference's own setup code and check that the lowering reproduces the
committed ``*.spec.npz`` exactly, and that the mask-free problem builder used
for the 65-site general-interaction spec agrees with the reference's full
``factorized_cc_problem`` where both run.  They need the reference package's
source tree next to this repository and skip without it.
"""

from __future__ import annotations

import sys

import numpy as np
import pytest

from conftest import GOLDEN, ROOT

REFERENCE_SRC = ROOT.parent / "reference" / "src"
pytestmark = pytest.mark.skipif(not (REFERENCE_SRC / "c3l").is_dir(), reason="reference source tree not present")

# fixtures whose reference setup takes seconds (the 27-site Kanamori builds cluster masks for ~1 min)
SMALL = ("readme", "s135fix", "twosrc", "siam10", "kanamori3x2", "gen5x1")


@pytest.fixture(scope="module")
def mf():
    if str(REFERENCE_SRC) not in sys.path:
        sys.path.insert(0, str(REFERENCE_SRC))
    sys.path.insert(0, str(GOLDEN))
    import make_fixtures

    return make_fixtures


def _same(a: dict, b: dict) -> list:
    return [k for k in a if k != "recipe" and not np.array_equal(np.asarray(a[k]), np.asarray(b[k]))]


@pytest.mark.parametrize("name", SMALL)
def test_from_reference_reproduces_committed_spec(mf, name):
    from c3l.cc.component_tensor import ComponentStaticProblem as RefStatic

    import c3lindblad_gb300 as c3

    fx = mf.FIXTURES[name]
    cc = mf.build_problem(fx)
    committed = dict(np.load(GOLDEN / f"{name}.spec.npz"))
    # the reference's ComponentStaticProblem, as a user of the reference holds it
    ref_static = RefStatic.compile(cc)
    lowered = c3.ProblemSpec.from_reference(ref_static, fx["recipe"]).as_dict()
    assert _same(lowered, committed) == []
    # and the package's own entry point accepts both reference objects
    for obj in (cc, ref_static):
        mine = c3.ComponentStaticProblem.compile(obj)
        assert _same(mine.spec.as_dict(), committed) == []
        assert mine.oracle is cc


@pytest.mark.parametrize("name", ("gen5x1", "kanamori3x2"))
def test_mask_free_builder_matches_factorized_problem(mf, name):
    import c3lindblad_gb300 as c3

    fx = mf.FIXTURES[name]
    full = c3.ProblemSpec.from_factorized(mf.build_problem(fx), fx["recipe"]).as_dict()
    model, reference = mf.build_reference(fx)
    light = c3.ProblemSpec.from_factorized(mf.light_problem(model, reference), fx["recipe"]).as_dict()
    assert _same(full, light) == []


def test_general_interaction_65_site_spec_is_reproducible(mf):
    import c3lindblad_gb300 as c3

    fx = mf.SPEC_ONLY["gen5x12"]
    model, reference = mf.build_reference(fx)
    light = c3.ProblemSpec.from_factorized(mf.light_problem(model, reference), fx["recipe"]).as_dict()
    committed = dict(np.load(GOLDEN / "gen5x12.spec.npz"))
    assert _same(light, committed) == []
    assert int(light["n"]) == 65
    lengths = np.asarray(light["product_lengths"])
    assert int(np.sum(lengths == 4)) == 1650 and int(np.sum(lengths == 2)) == 100
