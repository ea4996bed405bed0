"""The compiled device tables reproduce the reference (checked on CPU).

``plan_interpreter`` executes the exact tables the CUDA kernels consume, so
these tests pin the symbolic compiler, the coordinate layout and the tilde
tables without a GPU.
"""

from __future__ import annotations

import ctypes

import numpy as np
import pytest

from conftest import eom_amplitudes, golden_names, load, relerr
from c3lindblad_gb300 import compiler, layout
from c3lindblad_gb300.plans import EOMPlan, StaticPlan
from oracle import component_oracle as oc
from plan_interpreter import InterpretedEOM, InterpretedStatic, run_canonical, run_pairs


@pytest.fixture(scope="module")
def plans():
    cache = {}

    def get(name):
        if name not in cache:
            spec, g = load(name)
            cache[name] = (spec, g, StaticPlan(spec))
        return cache[name]

    return get


@pytest.mark.parametrize("name", golden_names())
def test_layout_matches_reference_order(name):
    spec, g = load(name)
    c = layout.static_coordinates(spec.n)
    if "cluster_masks" in g:
        masks = np.where(c.modes >= 0, np.left_shift(1, np.maximum(c.modes, 0)), 0).sum(axis=1)
        assert np.array_equal(masks, g["cluster_masks"])
    tl = layout.tilde_layout(c, spec.mode_partner, spec.mode_phase)
    assert np.array_equal(tl.partner, g["tilde_partner"])
    assert np.allclose(tl.phase, g["tilde_phase"], atol=1e-14)
    assert np.array_equal(tl.rep_pos, g["tilde_independent"])
    x = g["fixed_variables"]
    assert np.allclose(tl.coef_a * x[tl.idx_a] + tl.coef_b * x[tl.idx_b], g["fixed_amplitudes"], atol=1e-18, rtol=0)


@pytest.mark.parametrize("n", [1, 2, 3, 4, 5])
def test_layout_masks_small_n(n):
    c = layout.static_coordinates(n)
    m = np.where(c.modes >= 0, np.left_shift(1, np.maximum(c.modes, 0)), 0).sum(axis=1)
    assert list(m) == oc.static_masks(n)
    assert c.dimension == layout.amplitude_count(n)
    for spin in (0, 1):
        for charge in (1, -1):
            e = layout.eom_coordinates(n, spin, charge)
            m = np.where(e.modes >= 0, np.left_shift(1, np.maximum(e.modes, 0)), 0).sum(axis=1)
            assert list(m) == oc.eom_masks(n, spin, charge)


@pytest.mark.parametrize("name", golden_names())
def test_compiled_residual_and_jvp(name, plans):
    spec, g, plan = plans(name)
    it = InterpretedStatic(plan)
    tilde = oc.Tilde(oc.static_masks(spec.n), spec.mode_partner, spec.mode_phase) if spec.n <= 11 else None
    r, ref = it.residual(g["fixed_variables"], linearize=True)
    packed = np.empty(plan.num_variables)
    t = plan.tilde
    packed[t.rep_col] = (g["residual"][t.rep_pos] * t.rep_scale).real
    pr = t.rep_pair == 1
    packed[t.rep_col[pr] + 1] = g["residual"][t.rep_pos[pr]].imag
    assert relerr(r, packed) < 1e-12
    assert abs(ref - g["residual_reference"]) < 1e-12 * max(1.0, abs(g["residual_reference"]))
    j, jref = it.jvp(g["fixed_direction_variables"])
    packed[t.rep_col] = (g["jvp"][t.rep_pos] * t.rep_scale).real
    packed[t.rep_col[pr] + 1] = g["jvp"][t.rep_pos[pr]].imag
    assert relerr(j, packed) < 1e-12
    assert abs(jref - g["jvp_reference"]) < 1e-12 * max(1.0, abs(g["jvp_reference"]))


@pytest.mark.parametrize("name", golden_names())
def test_pair_gemm_stage_matches_instance_stage(name, plans):
    """The GEMM form of the JVP output (pair GEMMs + gather) equals the
    instance form on the same workspace, and so the reference's JVP."""
    spec, g, plan = plans(name)
    it = InterpretedStatic(plan)
    it.residual(g["fixed_variables"], linearize=True)
    it.jvp(g["fixed_direction_variables"])
    prog = plan.program
    for stage in ("res", "jvp"):  # the residual's stage reads the same workspace
        want = run_canonical(prog, stage, it.ws)
        got = run_canonical(prog, f"{stage}_pairs", run_pairs(prog, stage, it.ws))
        assert relerr(got, want) < 1e-13
        pp = prog.pairs[stage]
        assert pp.size <= prog.pair_size and pp.tiles["group"].max() == pp.groups.size - 1
        # every tile lies inside its group's P block, every block inside the buffer
        gr = pp.groups[pp.tiles["group"]]
        assert np.all(pp.tiles["m0"] < gr["M"]) and np.all(pp.tiles["n0"] < gr["N"])
        assert np.all(pp.groups["p_off"] + pp.groups["M"].astype(np.int64) * pp.groups["N"] <= prog.pair_size)
        assert np.all(pp.aoff >= 0) and np.all(pp.roff >= 0) and np.all(pp.aoff < prog.ws_size)


@pytest.mark.parametrize("name", golden_names(with_eom=True))
@pytest.mark.parametrize("charge", [1, -1])
def test_sigma_pair_gemm_stage_matches_instance_stage(name, charge, plans):
    spec, g, plan = plans(name)
    tag = "p" if charge == 1 else "m"
    ep = EOMPlan(plan, 0, charge)
    it = InterpretedEOM(ep, eom_amplitudes(g))
    it.sigma(g[f"eom{tag}_probe"])
    prog = ep.program
    want = run_canonical(prog, "sigma", it.ws)
    got = run_canonical(prog, "sigma_pairs", run_pairs(prog, "sigma", it.ws))
    assert relerr(got, want) < 1e-13


@pytest.mark.parametrize("name", golden_names(with_eom=True))
@pytest.mark.parametrize("charge", [1, -1])
def test_compiled_sigma_and_sources(name, charge, plans):
    spec, g, plan = plans(name)
    tag = "p" if charge == 1 else "m"
    ep = EOMPlan(plan, 0, charge)
    it = InterpretedEOM(ep, eom_amplitudes(g))
    assert relerr(ep.diagonal, g[f"eom{tag}_diagonal"]) < 1e-14
    assert relerr(it.sigma(g[f"eom{tag}_probe"]), g[f"eom{tag}_sigma"]) < 1e-12
    add, rem, sink = it.sources(spec.impurity_site)
    assert np.max(np.abs(add - g[f"eom{tag}_addition"])) < 1e-12
    assert np.max(np.abs(rem - g[f"eom{tag}_removal"])) < 1e-12
    assert np.max(np.abs(sink - g[f"eom{tag}_sink"])) < 1e-14


def test_program_table_layouts_match_c_structs():
    """NumPy structured dtypes mirror the C structs of include/c3l_gb300.h."""

    class Task(ctypes.Structure):
        _fields_ = [("dst_off", ctypes.c_int64), ("deg", ctypes.c_int32), ("nsrc", ctypes.c_int32),
                    ("const_off", ctypes.c_int64), ("src_off", ctypes.c_int64 * 4), ("vec_off", ctypes.c_int64 * 4),
                    ("axis", ctypes.c_int32 * 4), ("sign", ctypes.c_double * 4)]

    class Inst(ctypes.Structure):
        _fields_ = [("coef", ctypes.c_double * 2), ("nfac", ctypes.c_int32), ("pad", ctypes.c_int32),
                    ("fac_off", ctypes.c_int64 * 6), ("fac_deg", ctypes.c_int32 * 6), ("axes", (ctypes.c_int8 * 6) * 6)]

    class Block(ctypes.Structure):
        _fields_ = [("inst_begin", ctypes.c_int64), ("inst_end", ctypes.c_int64), ("out_off", ctypes.c_int64),
                    ("deg", ctypes.c_int32), ("pad", ctypes.c_int32)]

    class Tile(ctypes.Structure):
        _fields_ = [("block", ctypes.c_int32), ("count", ctypes.c_int32), ("start", ctypes.c_int64)]

    class PairGroup(ctypes.Structure):
        _fields_ = [("p_off", ctypes.c_int64), ("kbegin", ctypes.c_int64), ("kend", ctypes.c_int64),
                    ("M", ctypes.c_int32), ("N", ctypes.c_int32)]

    class PairTile(ctypes.Structure):
        _fields_ = [("group", ctypes.c_int32), ("m0", ctypes.c_int32), ("n0", ctypes.c_int32), ("shape", ctypes.c_int32)]

    for dt, cs in ((compiler.CONTRACT_DTYPE, Task), (compiler.INSTANCE_DTYPE, Inst),
                   (compiler.BLOCK_DTYPE, Block), (compiler.TILE_DTYPE, Tile),
                   (compiler.PAIR_GROUP_DTYPE, PairGroup), (compiler.PAIR_TILE_DTYPE, PairTile)):
        assert dt.itemsize == ctypes.sizeof(cs)
        for name, *_ in cs._fields_:
            assert dt.fields[name][1] == getattr(cs, name).offset, name


def test_multi_shuffle_signs_match_pairwise_wedge():
    """Iterated shuffles equal the reference's pairwise block wedge signs."""
    rng = np.random.default_rng(3)
    n = 3
    keys = [(1, 0, 1, 0), (0, 1, 0, 0), (1, 0, 0, 1)]
    arrays = [rng.normal(size=(n,) * sum(k)) + 1j * rng.normal(size=(n,) * sum(k)) for k in keys]
    out_key = tuple(sum(k[g] for k in keys) for g in range(4))
    ref = oc.wedge_blocks(arrays[0], keys[0], arrays[1], keys[1], n)
    ref = oc.wedge_blocks(ref, oc.add_key(keys[0], keys[1]), arrays[2], keys[2], n)
    got = np.zeros((n,) * sum(out_key), complex)
    for idx in np.ndindex(*got.shape):
        acc = 0j
        for sign, lists in compiler.multi_shuffles(out_key, keys):
            v = sign
            for a, lst in zip(arrays, lists):
                v = v * a[tuple(idx[ax] for ax in lst)]
            acc += v
        got[idx] = acc
    assert np.allclose(got, ref, atol=1e-13)


@pytest.mark.parametrize("M,N,K", [(1, 1, 1), (65, 65, 9), (27, 729, 40), (729, 27, 3), (4225, 65, 20),
                                   (65, 274625, 10), (19683, 1, 6), (4225, 1, 200), (11, 121, 5)])
def test_pair_tiles_cover_each_entry_once(M, N, K):
    """The CUDA-core tiles of a pair group cover its M x N entries exactly once
    and pick the least padded shape (one-column groups: the column tiles)."""
    tiles = compiler.pair_tiles(M, N, K)
    hit = np.zeros((M, N), np.int32)
    for m0, n0, shape in tiles:
        if shape in compiler.PAIR_COLUMN_ROWS:
            assert N == 1
            tm, tn = compiler.PAIR_COLUMN_ROWS[shape], 1
            assert (shape == compiler.PAIR_COLUMN_SPLIT) == (K >= compiler.PAIR_COLUMN_SPLIT_MIN)
        else:
            tm, tn = compiler.PAIR_SHAPES[shape]
        hit[m0:m0 + tm, n0:n0 + tn] += 1
    assert np.all(hit == 1)
    if N > 1:
        shape = tiles[0][2]
        tm, tn = compiler.PAIR_SHAPES[shape]
        area = len(tiles) * tm * tn
        assert area == min(-(-M // a) * a * (-(-N // b) * b) for a, b in compiler.PAIR_SHAPES.values())
