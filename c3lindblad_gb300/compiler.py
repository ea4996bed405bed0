"""Symbolic compilation of factorized products into flat device programs.

The reference evaluates each product ``c * F_1 ... F_m |0>`` with transformed
factors ``F + [F, T] = creator ^ . + (iota_a T) ^ . + iota_a`` on lazy term
lists of padded blocks (``src/c3l/cc/component_tensor.py:764-786`` and
``:1166-1233``).  The structure of those term lists does not depend on the
site count n, so this module expands it once, symbolically, and emits tables
that a handful of generic GPU kernels execute.

Atoms
    An atom is a homogeneous exterior form obtained from a *base* by a chain
    of interior products with factor annihilators (applied in order):

    * ``B1(f, src)`` = creator(f) + iota_f src_2   (degree 1; the creator only
      for the amplitudes ``T``, not for a tangent ``V``),
    * ``B3(f, src)`` = iota_f src_4                (degree 3),
    * ``X(d)``       = degree-d part of an EOM response vector.

    Merging the creator with the degree-one shift is exact: both are wedged
    and contracted identically (the reference keeps them as separate terms).

Monomials
    A term is ``coef * atom_1 ^ atom_2 ^ ...``; degree-zero atoms are scalars.
    Terms are canonicalized (graded sort with signs) and merged.  For each
    term the highest-degree atom (variable sources first) is the *anchor* and
    the rest of the wedge is summed per anchor into a *rest form*:

        out = sum_anchor anchor ^ rest_anchor,
        rest_anchor = sum_terms coef * scalars * (wedge of the other atoms).

    Both sums are evaluated by one generic kernel that sums shuffle-signed
    products of padded block entries ("instances") per output element.

Tables
    ``ContractTask`` rows build atoms; ``Instance`` rows drive the wedge
    evaluator; ``Tile`` rows split outputs into thread blocks.  All are
    NumPy structured arrays with the exact layout of the C structs in
    ``include/c3l_gb300.h``.
"""

from __future__ import annotations

from collections import defaultdict
from dataclasses import dataclass, field
from itertools import combinations, product

import numpy as np

from .layout import Coordinates

MAX_FACTORS = 6
MAX_DEGREE = 6   # index digits per output (C3L_MAX_DEGREE): static and S13 need 4, S135 5
MAX_SOURCES = 4
TILE = 256        # outputs per contraction tile (one thread each)
WEDGE_WIDTHS = (64, 32, 16, 8)  # outputs per wedge tile; a block of 256 threads splits
                                # each output's instances over 256 / width thread groups
WEDGE_MIN_TILES = 608           # narrowest width reaching this many tiles (4 per GB300 SM)

CONTRACT_DTYPE = np.dtype([
    ("dst_off", np.int64), ("deg", np.int32), ("nsrc", np.int32),
    ("const_off", np.int64),
    ("src_off", np.int64, (MAX_SOURCES,)), ("vec_off", np.int64, (MAX_SOURCES,)),
    ("axis", np.int32, (MAX_SOURCES,)), ("sign", np.float64, (MAX_SOURCES,)),
], align=True)

INSTANCE_DTYPE = np.dtype([
    ("coef", np.float64, (2,)), ("nfac", np.int32), ("pad", np.int32),
    ("fac_off", np.int64, (MAX_FACTORS,)), ("fac_deg", np.int32, (MAX_FACTORS,)),
    ("axes", np.int8, (MAX_FACTORS, MAX_DEGREE)),
], align=True)

BLOCK_DTYPE = np.dtype([
    ("inst_begin", np.int64), ("inst_end", np.int64), ("out_off", np.int64),
    ("deg", np.int32), ("pad", np.int32),
], align=True)

TILE_DTYPE = np.dtype([("block", np.int32), ("count", np.int32), ("start", np.int64)], align=True)

# Pair GEMMs of an output stage: group g computes P_g[i, j] = sum_k A_k[i] R_k[j]
# over its anchors k (rows aoff[k] .. + M and roff[k] .. + N of the workspace),
# P_g row-major M x N at offset p_off of the pair buffer that follows the workspace.
PAIR_GROUP_DTYPE = np.dtype([("p_off", np.int64), ("kbegin", np.int64), ("kend", np.int64),
                             ("M", np.int32), ("N", np.int32)], align=True)
PAIR_TILE_DTYPE = np.dtype([("group", np.int32), ("m0", np.int32), ("n0", np.int32), ("shape", np.int32)],
                           align=True)
PAIR_TILE = 64    # P entries per side of the default CUDA-core tile
PAIR_TILE_TC = (128, 64)  # tensor-core tiles: rows (tensor-memory lanes) x columns
# CUDA-core tile shapes (c3l_pair_tile.shape, C3L_PAIR_SHAPE_*): rows x columns,
# in order of preference when several pad a group equally
PAIR_SHAPES = {0: (64, 64), 1: (32, 128), 2: (128, 32), 3: (16, 256), 4: (256, 16)}
PAIR_COLUMN, PAIR_COLUMN_SPLIT = 5, 6      # one-column groups: 256 rows / 32 rows, anchors split by warps
PAIR_COLUMN_ROWS = {PAIR_COLUMN: 256, PAIR_COLUMN_SPLIT: 32}
PAIR_COLUMN_SPLIT_MIN = 16                 # anchors from which the column tiles split them


def pair_tiles(M: int, N: int, K: int) -> list:
    """CUDA-core tiles (m0, n0, shape) of one pair group of M x N entries and K anchors.

    One-column groups (N = 1) are matrix-vector products: 256-row tiles with
    one row per thread, or, from PAIR_COLUMN_SPLIT_MIN anchors on, 32-row
    tiles whose 8 warps split the anchors.  Every other group takes the
    rectangular shape that pads it least (a group of 27 rows fills a
    32 x 128 tile to 84 %, a 64 x 64 one to 42 %).
    """
    if N == 1:
        shape = PAIR_COLUMN_SPLIT if K >= PAIR_COLUMN_SPLIT_MIN else PAIR_COLUMN
        return [(m0, 0, shape) for m0 in range(0, M, PAIR_COLUMN_ROWS[shape])]

    def padded(s):
        tm, tn = PAIR_SHAPES[s]
        return -(-M // tm) * tm * (-(-N // tn) * tn)

    shape = min(PAIR_SHAPES, key=lambda s: (padded(s), s))
    tm, tn = PAIR_SHAPES[shape]
    return [(m0, n0, shape) for m0 in range(0, M, tm) for n0 in range(0, N, tn)]


def _e(g: int) -> tuple:
    return tuple(1 if h == g else 0 for h in range(4))


def _sub(a, b):
    return tuple(x - y for x, y in zip(a, b))


def _add(a, b):
    return tuple(x + y for x, y in zip(a, b))


@dataclass(frozen=True, order=True)
class Atom:
    src: str          # "T", "V" (static tangent) or "X" (EOM response)
    f: int            # factor index; -1 for X
    part: int         # degree of the base
    chain: tuple = () # factors contracted in order

    @property
    def degree(self) -> int:
        return self.part - len(self.chain)

    def contract(self, g: int) -> "Atom":
        return Atom(self.src, self.f, self.part, self.chain + (g,))


SRC_RANK = {"V": 0, "X": 0, "T": 1}


def _atom_sort_key(a: Atom):
    return (-a.degree, SRC_RANK[a.src], a.f, a.part, a.chain)


def _odd_inversions(seq) -> bool:
    odd = False
    for i in range(len(seq)):
        for j in range(i + 1, len(seq)):
            if seq[i] > seq[j]:
                odd = not odd
    return odd


def multi_shuffles(out_key: tuple, keys: list):
    """All axis assignments of a multi-factor block wedge and their signs.

    Output axes are group-major; factor j receives ``keys[j][g]`` axes of
    group g, in increasing order.  The sign is the parity of the
    concatenated factor axis lists -- the iterated form of
    ``src/c3l/cc/component_tensor.py:63-79``.
    """
    starts = np.cumsum((0,) + tuple(out_key))
    per_group = []
    for g in range(4):
        axes = list(range(int(starts[g]), int(starts[g + 1])))
        sizes = [k[g] for k in keys]
        assignments = []

        def rec(remaining, j, acc):
            if j == len(sizes):
                if not remaining:
                    assignments.append(list(acc))
                return
            for pick in combinations(remaining, sizes[j]):
                rest = [a for a in remaining if a not in pick]
                rec(rest, j + 1, acc + [list(pick)])

        rec(axes, 0, [])
        per_group.append(assignments)
    for choice in product(*per_group):
        lists = [[ax for g in range(4) for ax in choice[g][j]] for j in range(len(keys))]
        flat = [ax for lst in lists for ax in lst]
        yield (-1.0 if _odd_inversions(flat) else 1.0), lists


class Symbolic:
    """Block-structure bookkeeping and term expansion for one problem."""

    def __init__(self, spec, static_coords: Coordinates, eom_keys=()):
        self.n = n = spec.n
        cre = np.asarray(spec.creators)
        ann = np.asarray(spec.annihilators)
        self.F = cre.shape[0]
        self.cre_groups = [tuple(g for g in range(4) if np.any(cre[f, g * n:(g + 1) * n])) for f in range(self.F)]
        self.ann_groups = [tuple(g for g in range(4) if np.any(ann[f, g * n:(g + 1) * n])) for f in range(self.F)]
        skeys = list(static_coords.keys)
        self.source_keys = {
            "T": {2: frozenset(k for k in skeys if sum(k) == 2), 4: frozenset(k for k in skeys if sum(k) == 4)},
            "V": {2: frozenset(k for k in skeys if sum(k) == 2), 4: frozenset(k for k in skeys if sum(k) == 4)},
            "X": {d: frozenset(k for k in eom_keys if sum(k) == d) for d in (1, 3, 5)},
        }
        self._blocks: dict = {}

    # -------------------------------------------------------------- blocks
    def _contract_keys(self, keys, g: int):
        out = set()
        for k in keys:
            for h in self.ann_groups[g]:
                if k[h] > 0:
                    out.add(_sub(k, _e(h)))
        return frozenset(out)

    def blocks(self, a: Atom) -> frozenset:
        got = self._blocks.get(a)
        if got is not None:
            return got
        if a.chain:
            res = self._contract_keys(self.blocks(Atom(a.src, a.f, a.part, a.chain[:-1])), a.chain[-1])
        elif a.src == "X":
            res = self.source_keys["X"][a.part]
        else:
            base = self._contract_keys(self.source_keys[a.src][a.part + 1], a.f)
            if a.part == 1 and a.src == "T":
                base = base | frozenset(_e(g) for g in self.cre_groups[a.f])
            res = base
        self._blocks[a] = res
        return res

    def nonzero(self, a: Atom) -> bool:
        return a.degree >= 0 and bool(self.blocks(a))

    # ----------------------------------------------------------- expansion
    @staticmethod
    def canonical(coef: complex, atoms: tuple):
        """Graded sort of the non-scalar atoms; scalars sorted freely."""
        scal = sorted(a for a in atoms if a.degree == 0)
        non = [a for a in atoms if a.degree > 0]
        sign = 1.0
        # bubble sort with graded transposition signs
        changed = True
        while changed:
            changed = False
            for i in range(len(non) - 1):
                if _atom_sort_key(non[i + 1]) < _atom_sort_key(non[i]):
                    if (non[i].degree * non[i + 1].degree) % 2:
                        sign = -sign
                    non[i], non[i + 1] = non[i + 1], non[i]
                    changed = True
        return coef * sign, tuple(non) + tuple(scal)

    def apply_factor(self, states, f: int):
        """Transformed factor on lazy terms (component_tensor.py:764-786)."""
        out = []
        wedges = [a for a in (Atom("T", f, 1), Atom("T", f, 3)) if self.nonzero(a)]
        has_ann = bool(self.ann_groups[f])
        for coef, atoms in states:
            for w in wedges:
                out.append((coef, (w,) + atoms))
            if has_ann:
                prefix = 0
                for pos, a in enumerate(atoms):
                    if a.degree > 0:
                        b = a.contract(f)
                        if self.nonzero(b):
                            out.append((coef * (-1) ** prefix, atoms[:pos] + (b,) + atoms[pos + 1:]))
                    prefix += a.degree
        return out

    def expand(self, products, init: tuple, max_out: int, keep: set):
        """All monomials of ``sum_p c_p F_1..F_m init |0>`` with degree in ``keep``."""
        acc: dict = defaultdict(complex)
        for coef, facs in products:
            states = [(coef, init)]
            m = len(facs)
            for step, f in enumerate(reversed(facs)):
                remaining = m - step - 1
                states = [(c, a) for c, a in self.apply_factor(states, f)
                          if sum(x.degree for x in a) - remaining <= max_out]
            for c, atoms in states:
                if sum(x.degree for x in atoms) in keep:
                    cc, ca = self.canonical(c, atoms)
                    acc[ca] += cc
        return {k: v for k, v in acc.items() if v != 0}

    def differentiate(self, terms: dict, var: str = "V"):
        """Product rule: replace one amplitude atom at a time by its tangent."""
        acc: dict = defaultdict(complex)
        for atoms, coef in terms.items():
            for j, a in enumerate(atoms):
                if a.src != "T":
                    continue
                d = Atom(var, a.f, a.part, a.chain)
                if not self.nonzero(d):
                    continue
                cc, ca = self.canonical(coef, atoms[:j] + (d,) + atoms[j + 1:])
                acc[ca] += cc
        return {k: v for k, v in acc.items() if v != 0}


# ====================================================================== plan
@dataclass
class Stage:
    """One wedge-evaluation launch: output blocks, their instances and tiles."""

    name: str
    kind: str                 # "padded" or "canonical"
    blocks: np.ndarray        # BLOCK_DTYPE
    instances: np.ndarray     # INSTANCE_DTYPE
    tiles: np.ndarray         # TILE_DTYPE
    elements: np.ndarray | None = None   # canonical: int64 vector positions
    digits: np.ndarray | None = None     # canonical: int32 packed index digits
    element_block: np.ndarray | None = None
    width: int = 64                      # outputs per tile
    pair_relative: bool = False          # instance offsets count from the pair buffer (fixed in finish)


@dataclass
class PairProgram:
    """The GEMMs feeding a ``<name>_pairs`` gather stage (offsets into the pair buffer)."""

    groups: np.ndarray        # PAIR_GROUP_DTYPE
    aoff: np.ndarray          # int64 workspace offsets of anchor rows
    roff: np.ndarray          # int64 workspace offsets of rest rows
    tiles: np.ndarray         # PAIR_TILE_DTYPE (PAIR_TILE x PAIR_TILE)
    size: int                 # pair-buffer entries
    tiles_tc: np.ndarray | None = None  # PAIR_TILE_DTYPE (PAIR_TILE_TC)

    @property
    def macs(self) -> int:
        g = self.groups
        return int(np.sum((g["kend"] - g["kbegin"]) * g["M"].astype(np.int64) * g["N"].astype(np.int64)))


@dataclass
class ContractLevel:
    tasks: np.ndarray         # CONTRACT_DTYPE
    tiles: np.ndarray         # TILE_DTYPE


@dataclass
class Program:
    n: int
    ws_size: int
    vectors: np.ndarray                       # complex [*]: factor creator/annihilator group vectors
    source_offsets: dict                      # src -> {key: ws offset}
    levels: dict = field(default_factory=dict)   # class -> [ContractLevel]
    stages: dict = field(default_factory=dict)   # name -> Stage
    atom_offsets: dict = field(default_factory=dict)
    rest_offsets: dict = field(default_factory=dict)
    pairs: dict = field(default_factory=dict)    # stage name -> PairProgram
    pair_size: int = 0                           # pair-buffer entries (after the workspace): the largest program


class Builder:
    """Lays out the workspace and emits the device tables."""

    def __init__(self, sym: Symbolic, spec):
        self.sym = sym
        self.n = sym.n
        self.ws = 0
        self.source_offsets: dict = {}
        self.atom_offsets: dict = {}
        self.rest_offsets: dict = {}
        n = self.n
        cre = np.asarray(spec.creators)
        ann = np.asarray(spec.annihilators)
        F = cre.shape[0]
        # vectors table: [F][kind(0=creator,1=annihilator)][group][n]
        self.vectors = np.zeros((F, 2, 4, n), np.complex128)
        for f in range(F):
            for g in range(4):
                self.vectors[f, 0, g] = cre[f, g * n:(g + 1) * n]
                self.vectors[f, 1, g] = ann[f, g * n:(g + 1) * n]
        self.levels: dict = defaultdict(lambda: defaultdict(list))
        self.stage_data: dict = {}
        self.pairs: dict = {}
        self.pair_size = 0

    def vec_off(self, f: int, kind: int, g: int) -> int:
        return ((f * 2 + kind) * 4 + g) * self.n

    def alloc(self, key: tuple) -> int:
        off = self.ws
        self.ws += self.n ** sum(key)
        return off

    def add_source(self, src: str, keys) -> None:
        self.source_offsets[src] = {k: self.alloc(k) for k in sorted(keys)}

    # ------------------------------------------------------------- atoms
    def atom_class(self, a: Atom) -> str:
        return a.src

    def ensure_atom(self, a: Atom) -> dict:
        """Allocate (and emit contraction tasks for) an atom and its parents."""
        got = self.atom_offsets.get(a)
        if got is not None:
            return got
        sym = self.sym
        if a.src == "X" and not a.chain:
            offs = {k: self.source_offsets["X"][k] for k in sym.blocks(a)}
            self.atom_offsets[a] = offs
            return offs
        if a.chain:
            parent = Atom(a.src, a.f, a.part, a.chain[:-1])
            pof = self.ensure_atom(parent)
            g = a.chain[-1]
            level = len(a.chain)
        else:
            parent = None
            pof = self.source_offsets[a.src]
            g = a.f
            level = 0
        offs = {}
        for k in sorted(sym.blocks(a)):
            offs[k] = self.alloc(k)
        for k, dst in offs.items():
            srcs = []
            for h in sym.ann_groups[g]:
                sk = _add(k, _e(h))
                if parent is None:
                    valid = sk in sym.source_keys[a.src][a.part + 1]
                else:
                    valid = sk in sym.blocks(parent)
                if not valid:
                    continue
                axis = sum(sk[:h])
                srcs.append((pof[sk], self.vec_off(g, 1, h), axis, (-1.0) ** axis))
            const = -1
            if parent is None and a.part == 1 and a.src == "T" and sum(k) == 1:
                gc = k.index(1)
                if gc in sym.cre_groups[a.f]:
                    const = self.vec_off(a.f, 0, gc)
            assert len(srcs) <= MAX_SOURCES
            self.levels[a.src][level].append((dst, sum(k), const, srcs))
        self.atom_offsets[a] = offs
        return offs

    # ------------------------------------------------------ wedge stages
    def rest_blocks(self, anchor: Atom, out_keys, terms) -> set:
        sym = self.sym
        need = set()
        for ko in out_keys:
            for ka in sym.blocks(anchor):
                kr = _sub(ko, ka)
                if min(kr) >= 0:
                    need.add(kr)
        possible = set()
        for (scal, rest), _ in terms.items():
            for choice in product(*[sorted(sym.blocks(a)) for a in rest]):
                s = (0, 0, 0, 0)
                for k in choice:
                    s = _add(s, k)
                possible.add(s)
        return need & possible

    def wedge_instances(self, out_key, coef, scal, atoms, atom_offs_fn):
        """Instances for ``coef * scalars * wedge(atoms)`` at one output block."""
        sym = self.sym
        rows = []
        soffs = [atom_offs_fn(s)[(0, 0, 0, 0)] for s in scal]
        for choice in product(*[sorted(sym.blocks(a)) for a in atoms]):
            s = (0, 0, 0, 0)
            for k in choice:
                s = _add(s, k)
            if s != tuple(out_key):
                continue
            for sign, lists in multi_shuffles(out_key, list(choice)):
                facs = [(atom_offs_fn(a)[k], sum(k), lst) for a, k, lst in zip(atoms, choice, lists)]
                facs += [(o, 0, []) for o in soffs]
                rows.append((coef * sign, facs))
        return rows

    def emit_stage(self, name: str, kind: str, block_rows, elements=None, digits=None, element_block=None):
        """block_rows: list of (out_off, deg, [instances]) in output order."""
        nb = len(block_rows)
        blocks = np.zeros(nb, BLOCK_DTYPE)
        inst_list = []
        for b, (out_off, deg, rows) in enumerate(block_rows):
            blocks[b]["inst_begin"] = len(inst_list)
            inst_list.extend(rows)
            blocks[b]["inst_end"] = len(inst_list)
            blocks[b]["out_off"] = out_off
            blocks[b]["deg"] = deg
        inst = np.zeros(len(inst_list), INSTANCE_DTYPE)
        for i, (coef, facs) in enumerate(inst_list):
            assert len(facs) <= MAX_FACTORS, len(facs)
            inst[i]["coef"] = (coef.real, coef.imag)
            inst[i]["nfac"] = len(facs)
            inst[i]["axes"] = -1
            for j, (off, deg, lst) in enumerate(facs):
                inst[i]["fac_off"][j] = off
                inst[i]["fac_deg"][j] = deg
                for q, ax in enumerate(lst):
                    inst[i]["axes"][j][q] = ax
        if kind == "padded":
            ranges = [(b, 0, self.n ** deg) for b, (out_off, deg, rows) in enumerate(block_rows)]
        else:
            eb = np.asarray(element_block)
            order_ok = np.all(np.diff(eb) >= 0)
            assert order_ok, "canonical elements must be grouped by block"
            ranges = []
            for b in range(nb):
                idx = np.flatnonzero(eb == b)
                if idx.size:
                    ranges.append((b, int(idx[0]), int(idx[-1]) + 1))
        width, tiles = _tiles_for(ranges)
        tarr = np.zeros(len(tiles), TILE_DTYPE)
        for i, (b, c, s) in enumerate(tiles):
            tarr[i] = (b, c, s)
        self.stage_data[name] = Stage(name, kind, blocks, inst, tarr, elements, digits, element_block, width)

    def finish(self) -> Program:
        levels = {}
        for cls, by_level in self.levels.items():
            lv = []
            for level in sorted(by_level):
                rows = by_level[level]
                tasks = np.zeros(len(rows), CONTRACT_DTYPE)
                tiles = []
                for i, (dst, deg, const, srcs) in enumerate(rows):
                    tasks[i]["dst_off"] = dst
                    tasks[i]["deg"] = deg
                    tasks[i]["nsrc"] = len(srcs)
                    tasks[i]["const_off"] = const
                    for j, (so, vo, ax, sg) in enumerate(srcs):
                        tasks[i]["src_off"][j] = so
                        tasks[i]["vec_off"][j] = vo
                        tasks[i]["axis"][j] = ax
                        tasks[i]["sign"][j] = sg
                    size = self.n ** deg
                    for s in range(0, size, TILE):
                        tiles.append((i, min(TILE, size - s), s))
                tarr = np.zeros(len(tiles), TILE_DTYPE)
                for i, t in enumerate(tiles):
                    tarr[i] = t
                lv.append(ContractLevel(tasks, tarr))
            levels[cls] = lv
        for st in self.stage_data.values():
            if st.pair_relative:
                nf = st.instances["nfac"]
                st.instances["fac_off"][nf > 0, 0] += self.ws
                st.pair_relative = False
        return Program(self.n, self.ws, self.vectors.reshape(-1), self.source_offsets, levels,
                       self.stage_data, self.atom_offsets, self.rest_offsets, self.pairs, self.pair_size)


def _tiles_for(ranges):
    """The widest tile that still gives every SM several blocks, and the tiles."""
    width = WEDGE_WIDTHS[-1]
    for w in WEDGE_WIDTHS:
        if sum(-(-(hi - lo) // w) for _, lo, hi in ranges) >= WEDGE_MIN_TILES:
            width = w
            break
    return width, [(b, min(width, hi - s), s) for b, lo, hi in ranges for s in range(lo, hi, width)]


def merge_padded(stages: list, n: int) -> "Stage":
    """One launch for several padded stages of an action.  Padded stages read
    atoms only and write disjoint workspace blocks, so their blocks can share
    a grid; the instance ranges and tile block indices are rebased."""
    blocks = np.concatenate([st.blocks for st in stages]).copy()
    inst = np.concatenate([st.instances for st in stages])
    b0 = i0 = 0
    for st in stages:
        nb = st.blocks.size
        blocks[b0:b0 + nb]["inst_begin"] += i0
        blocks[b0:b0 + nb]["inst_end"] += i0
        b0 += nb
        i0 += st.instances.size
    ranges = [(b, 0, n ** int(blocks[b]["deg"])) for b in range(blocks.size)]
    width, tiles = _tiles_for(ranges)
    tarr = np.zeros(len(tiles), TILE_DTYPE)
    for i, t in enumerate(tiles):
        tarr[i] = t
    return Stage("+".join(st.name for st in stages), "padded", blocks, inst, tarr, width=width)


def _group_by_anchor(terms: dict):
    """(anchor, out_degree) -> {(scalars, rest atoms): coef}; plus pure scalars."""
    groups: dict = defaultdict(lambda: defaultdict(complex))
    scalars: dict = defaultdict(complex)
    for atoms, coef in terms.items():
        non = [a for a in atoms if a.degree > 0]
        scal = tuple(a for a in atoms if a.degree == 0)
        D = sum(a.degree for a in non)
        if not non:
            scalars[scal] += coef
            continue
        anchor = non[0]
        groups[(anchor, D)][(scal, tuple(non[1:]))] += coef
    return groups, scalars


def _digits(coords: Coordinates, positions: np.ndarray) -> np.ndarray:
    """Index digits of each output packed one byte each, digit c in byte c
    (little-endian int64; padding digits are 0)."""
    tup = coords.tuples[positions]
    np.maximum(tup, 0, out=tup)
    packed = np.zeros((tup.shape[0], 8), np.uint8)
    packed[:, :tup.shape[1]] = tup  # every digit is below 256 (n <= 255)
    return packed.view("<i8").reshape(-1).astype(np.int64, copy=False)


def compile_output(builder: Builder, name: str, terms: dict, coords: Coordinates,
                   positions: np.ndarray, rest_stage: str, scalar_stage: str | None, extra=(), pairs: bool = False):
    """Emit rest stage(s) and the canonical output stage(s) for a term set.

    ``positions``: vector positions (in ``coords``) to evaluate, any order; the
    stage stores them grouped by block.  ``extra``: further canonical stages
    ``(stage_name, positions, scale)`` sharing the same rest forms, with every
    instance coefficient multiplied by ``scale``.  ``pairs``: also emit the
    GEMM form of the main stage (``compile_pairs``).  Returns the offset of the
    scalar (degree-zero) output in the workspace or -1.
    """
    sym = builder.sym
    groups, scalars = _group_by_anchor(terms)
    out_keys_by_deg = defaultdict(set)
    for k in coords.keys:
        out_keys_by_deg[sum(k)].add(k)
    # rest forms
    rest_rows_by_class = defaultdict(list)
    rest_info = {}
    for (anchor, D), rterms in sorted(groups.items(), key=lambda kv: (_atom_sort_key(kv[0][0]), kv[0][1])):
        out_keys = out_keys_by_deg.get(D, set())
        if not out_keys:
            continue
        blocks = builder.rest_blocks(anchor, out_keys, rterms)
        if not blocks:
            continue
        builder.ensure_atom(anchor)
        cls = "T"
        for (scal, rest) in rterms:
            for a in scal + rest:
                builder.ensure_atom(a)
                if a.src != "T":
                    cls = a.src
        offs = {k: builder.alloc(k) for k in sorted(blocks)}
        builder.rest_offsets[(name, anchor, D)] = offs
        rest_info[(anchor, D)] = offs
        for k in sorted(blocks):
            rows = []
            for (scal, rest), coef in rterms.items():
                rows.extend(builder.wedge_instances(k, coef, scal, rest, lambda a: builder.atom_offsets[a]))
            rest_rows_by_class[cls].append((offs[k], sum(k), rows))
    for cls, rows in rest_rows_by_class.items():
        builder.emit_stage(f"{rest_stage}_{cls}", "padded", rows)
    # scalar output
    scalar_off = -1
    if scalar_stage is not None and scalars:
        rows = []
        cls = "T"
        for scal, coef in scalars.items():
            for a in scal:
                builder.ensure_atom(a)
                if a.src != "T":
                    cls = a.src
            rows.extend(builder.wedge_instances((0, 0, 0, 0), coef, scal, (), lambda a: builder.atom_offsets[a]))
        scalar_off = builder.alloc((0, 0, 0, 0))
        builder.emit_stage(scalar_stage, "padded", [(scalar_off, 0, rows)])
    # canonical output(s)
    block_rows = []
    for b, key in enumerate(coords.keys):
        rows = []
        for (anchor, D), offs in rest_info.items():
            if D != sum(key):
                continue
            aoffs = builder.atom_offsets[anchor]
            for ka in sorted(sym.blocks(anchor)):
                kr = _sub(key, ka)
                if min(kr) < 0 or kr not in offs:
                    continue
                for sign, lists in multi_shuffles(key, [ka, kr]):
                    rows.append((complex(sign), [(aoffs[ka], sum(ka), lists[0]), (offs[kr], sum(kr), lists[1])]))
        block_rows.append((-1, sum(key), rows))
    for stage_name, stage_pos, scale in ((name, positions, 1.0),) + tuple(extra):
        pos = np.asarray(stage_pos, np.int64)
        blk = coords.block_of[pos]
        order = np.argsort(blk, kind="stable")
        pos = pos[order]
        blk = blk[order]
        rows_scaled = [(o, d, [(c * scale, f) for c, f in rows]) for o, d, rows in block_rows]
        builder.emit_stage(stage_name, "canonical", rows_scaled, elements=pos, digits=_digits(coords, pos),
                           element_block=blk)
        if pairs and stage_name == name:
            compile_pairs(builder, name, rest_info, coords, pos, blk)
    return scalar_off


def compile_pairs(builder: Builder, name: str, rest_info: dict, coords: Coordinates, pos: np.ndarray,
                  blk: np.ndarray) -> None:
    """GEMM form of a canonical output stage: stage ``<name>_pairs`` and ``builder.pairs[name]``.

    The stage's output at an element of block K is sum over anchors a and
    anchor blocks ka of shuffle-signed products A_a[ka](...) R_a[K - ka](...)
    (``compile_output``).  For fixed (K, ka) the shuffles do not depend on the
    anchor, so the products are first summed over the anchors as one padded
    GEMM P[i, j] = sum_a A_a[ka][i] R_a[K - ka][j] (i over n^|ka|, j over
    n^|K - ka| entries), and the element reads one signed entry of P per
    shuffle: a single-factor instance of degree |K| whose axes are the
    anchor's axes followed by the rest's.  The elements (and so the epilogue
    tables) are those of the instance stage, in the same order.
    """
    sym = builder.sym
    n = builder.n
    groups = []        # (block, ka, kr, [(aoff, roff)])
    for b, key in enumerate(coords.keys):
        by_ka: dict = defaultdict(list)
        for (anchor, D), offs in rest_info.items():
            if D != sum(key):
                continue
            aoffs = builder.atom_offsets[anchor]
            for ka in sorted(sym.blocks(anchor)):
                kr = _sub(key, ka)
                if min(kr) < 0 or kr not in offs:
                    continue
                by_ka[ka].append((aoffs[ka], offs[kr]))
        for ka in sorted(by_ka):
            groups.append((b, ka, _sub(key, ka), by_ka[ka]))
    garr = np.zeros(len(groups), PAIR_GROUP_DTYPE)
    aoff, roff, tiles = [], [], []
    block_rows = [(-1, sum(k), []) for k in coords.keys]
    p = 0  # every program's P blocks start at the pair buffer's first entry
    for g, (b, ka, kr, rows) in enumerate(groups):
        M, N = n ** sum(ka), n ** sum(kr)
        garr[g] = (p, len(aoff), len(aoff) + len(rows), M, N)
        aoff.extend(r[0] for r in rows)
        roff.extend(r[1] for r in rows)
        tiles.extend((g, m0, n0, shape) for m0, n0, shape in pair_tiles(M, N, len(rows)))
        key = coords.keys[b]
        for sign, lists in multi_shuffles(key, [ka, kr]):
            block_rows[b][2].append((complex(sign), [(p, sum(key), lists[0] + lists[1])]))
        p += M * N
    tarr = np.zeros(len(tiles), PAIR_TILE_DTYPE)
    for i, t in enumerate(tiles):
        tarr[i] = t
    tc = [(g, m0, n0, 0) for g, (b, ka, kr, rows) in enumerate(groups)
          for m0 in range(0, int(garr[g]["M"]), PAIR_TILE_TC[0]) for n0 in range(0, int(garr[g]["N"]), PAIR_TILE_TC[1])]
    tcarr = np.zeros(len(tc), PAIR_TILE_DTYPE)
    for i, t in enumerate(tc):
        tcarr[i] = t
    builder.pairs[name] = PairProgram(garr, np.asarray(aoff, np.int64), np.asarray(roff, np.int64), tarr, p, tcarr)
    builder.pair_size = max(builder.pair_size, p)
    builder.emit_stage(f"{name}_pairs", "canonical", block_rows, elements=pos, digits=_digits(coords, pos),
                       element_block=blk)
    builder.stage_data[f"{name}_pairs"].pair_relative = True


# ================================================================ front ends
def static_terms(sym: Symbolic, spec):
    """Residual monomials (degrees 0, 2, 4) and their tangents."""
    res = sym.expand(list(spec.products()), (), 4, {0, 2, 4})
    return res, sym.differentiate(res, "V")


def eom_terms(sym: Symbolic, spec, eom_keys, vacuum: dict):
    """Sigma monomials: products acting on X, minus vacuum ^ X (component_tensor.py:2116-2223);
    with rank-five keys, the full S135 action (``src/c3l/cc/s135_full.py:51-98``)."""
    acc: dict = defaultdict(complex)
    degs = sorted({sum(k) for k in eom_keys})
    keep = set(degs)  # {1, 3} for S13, {1, 3, 5} with the rank-five shell
    for d in degs:
        x = Atom("X", -1, d)
        if not sym.nonzero(x):
            continue
        part = sym.expand(list(spec.products()), (x,), max(degs), keep)
        for k, v in part.items():
            acc[k] += v
        for atoms, coef in vacuum.items():
            if sum(a.degree for a in atoms) + d not in keep:
                continue
            cc, ca = sym.canonical(-coef, atoms + (x,))
            acc[ca] += cc
    return {k: v for k, v in acc.items() if v != 0}
