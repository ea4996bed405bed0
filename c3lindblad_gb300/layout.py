"""Canonical coordinates, tilde orbits and padded-block index tables.

Everything here is vectorized NumPy setup work (no per-amplitude Python
loops), so it also scales to the large site counts where the reference's
mask enumeration is the bottleneck.

Vector order is the reference's: static amplitudes are sorted by
(particle-hole rank, bit mask) (``src/c3l/ci/basis.py:149-178`` and
``src/c3l/cc/factorized.py:332-338``); EOM coordinates of one spin/charge
follow ``response_basis`` (``src/c3l/ci/basis.py:181-236``) filtered to that
charge (``src/c3l/cc/component_tensor.py:2023``).  Sorting by the integer
mask of a fixed-rank mode set is colexicographic order of its ascending mode
tuple: highest mode first.

Inside a block the canonical index tuple is strictly increasing within
each group, and the device stores each block padded (``n**degree`` entries,
antisymmetric within groups) like ``ComponentCoordinates.unpack``
(``src/c3l/cc/component_tensor.py:302-325``).
"""

from __future__ import annotations

from dataclasses import dataclass
from itertools import combinations, permutations, product
from math import comb

import numpy as np

Key = tuple


def _combos(n: int, k: int) -> np.ndarray:
    if k == 0:
        return np.zeros((1, 0), np.int64)
    if k > n:
        return np.zeros((0, k), np.int64)
    return np.asarray(list(combinations(range(n), k)), np.int64).reshape(-1, k)


def block_tuples(n: int, key: Key) -> np.ndarray:
    """All canonical index tuples of one block, group-major, shape [count, degree]."""
    parts = [_combos(n, k) for k in key]
    sizes = [p.shape[0] for p in parts]
    total = int(np.prod(sizes))
    if total == 0:
        return np.zeros((0, sum(key)), np.int64)
    grids = np.indices(sizes).reshape(len(sizes), -1)
    cols = [parts[g][grids[g]] for g in range(4)]
    return np.concatenate(cols, axis=1)


def _modes(n: int, key: Key, tuples: np.ndarray) -> np.ndarray:
    offsets = np.concatenate([[g * n] * c for g, c in enumerate(key)]).astype(np.int64) if sum(key) else np.zeros(0, np.int64)
    return tuples + offsets[None, :]


@dataclass
class Coordinates:
    """Canonical coordinates of one vector space (static amplitudes or one EOM block)."""

    n: int
    keys: list            # block keys in sorted order
    block_of: np.ndarray  # int [D]  block id of each vector position
    tuples: np.ndarray    # int [D, dmax] canonical index tuple (group-major), -1 padded
    degree: np.ndarray    # int [D]
    modes: np.ndarray     # int [D, dmax] absolute modes ascending, -1 padded

    @property
    def dimension(self) -> int:
        return int(self.block_of.shape[0])

    def positions(self, key: Key) -> np.ndarray:
        return np.flatnonzero(self.block_of == self.keys.index(key))

    def rapidity_sum(self, rapidities: np.ndarray) -> np.ndarray:
        lam = np.concatenate([np.asarray(rapidities, np.complex128), [0.0]])
        return lam[self.modes].sum(axis=1)


def _ordered(n: int, rank_keys: list) -> Coordinates:
    """Build coordinates from (rank, key) pairs sorted by (rank, mask)."""
    dmax = max(sum(k) for _, k in rank_keys)
    recs_rank, recs_block, recs_tuple, recs_modes = [], [], [], []
    keys = sorted({k for _, k in rank_keys})
    for rank, key in rank_keys:
        t = block_tuples(n, key)
        if t.shape[0] == 0:
            continue
        m = _modes(n, key, t)
        d = sum(key)
        tp = -np.ones((t.shape[0], dmax), np.int64)
        tp[:, :d] = t
        mp = -np.ones((t.shape[0], dmax), np.int64)
        mp[:, :d] = np.sort(m, axis=1)
        recs_rank.append(np.full(t.shape[0], rank, np.int64))
        recs_block.append(np.full(t.shape[0], keys.index(key), np.int64))
        recs_tuple.append(tp)
        recs_modes.append(mp)
    rank = np.concatenate(recs_rank)
    block = np.concatenate(recs_block)
    tup = np.concatenate(recs_tuple)
    mod = np.concatenate(recs_modes)
    # colexicographic order of the ascending mode tuple within each rank:
    # primary key rank, then the highest mode, then the next highest, ...;
    # one integer key (modes + 1 < 2^bits, padding -1 -> 0) sorted stably
    bits = int(4 * n + 1).bit_length()
    if bits * dmax + int(rank.max()).bit_length() < 63:
        key = rank.astype(np.int64) << (bits * dmax)
        for c in range(dmax):
            key |= (mod[:, c] + 1) << (bits * c)
        order = np.argsort(key, kind="stable")
    else:
        order = np.lexsort([mod[:, c] for c in range(dmax)] + [rank])
    deg = np.asarray([sum(keys[b]) for b in block[order]], np.int64)
    return Coordinates(n, keys, block[order], tup[order], deg, mod[order])


def static_coordinates(n: int) -> Coordinates:
    """CCSD cluster coordinates: T1 keys (a,a,b,b) with a+b=1, T2 with a+b=2."""
    rk = []
    for rank in (1, 2):
        for a in range(rank + 1):
            b = rank - a
            if a <= n and b <= n:
                rk.append((rank, (a, a, b, b)))
    return _ordered(n, rk)


def eom_coordinates(n: int, spin: int, charge: int, space: str = "S13") -> Coordinates:
    """S13 coordinates of one response spin and charge; ``space="S135"``
    appends the rank-five shell.

    S13 is ordered like the reference's mask basis (``_ordered``).  The
    rank-five shell follows it block by block, in the reference's
    ``_charge_shell_keys`` order (keys of five creators with the response
    spin's charge, lexicographic over the four group counts) and, inside a
    block, row-major over each group's lexicographic index combinations
    (``ComponentCoordinateShell``, ``src/c3l/cc/component_tensor.py:384-559``).
    """
    if space not in ("S13", "S135"):
        raise ValueError("space must be 'S13' or 'S135'")
    rk = []
    for rank in (0, 1):
        for a in range(rank + 1):
            b = rank - a
            if a >= n or b > n:
                continue
            npl, nmi = (a + 1, a) if charge == 1 else (a, a + 1)
            key = (npl, nmi, b, b) if spin == 0 else (b, b, npl, nmi)
            rk.append((rank, key))
    base = _ordered(n, rk)
    if space == "S13":
        return base
    counts = range(min(n, 5) + 1)
    shell = [k for k in product(counts, counts, counts, counts)
             if sum(k) == 5 and (k[0] - k[1], k[2] - k[3]) == ((charge, 0) if spin == 0 else (0, charge))]
    keys = sorted(set(base.keys) | set(shell))
    remap = np.asarray([keys.index(k) for k in base.keys], np.int64)
    blocks, tuples, modes = [remap[base.block_of]], [], []
    dmax = 5
    pad = -np.ones((base.dimension, dmax - base.tuples.shape[1]), np.int64)
    tuples.append(np.concatenate([base.tuples, pad], axis=1))
    modes.append(np.concatenate([base.modes, pad], axis=1))
    for key in shell:
        t = block_tuples(n, key)
        if t.shape[0] == 0:
            continue
        blocks.append(np.full(t.shape[0], keys.index(key), np.int64))
        tuples.append(t)
        modes.append(np.sort(_modes(n, key, t), axis=1))
    block_of = np.concatenate(blocks)
    deg = np.asarray([sum(keys[b]) for b in block_of], np.int64)
    return Coordinates(n, keys, block_of, np.concatenate(tuples), deg, np.concatenate(modes))


# ------------------------------------------------------------------- tilde
@dataclass
class TildeLayout:
    """Tilde orbits of the static amplitudes and their real coordinates.

    ``t[mu] = coef_a[mu] * x[idx_a[mu]] + coef_b[mu] * x[idx_b[mu]]`` unpacks the
    independent real variables (``src/c3l/cc/symmetry.py:67-85``).  The
    residual is read back only at the orbit representatives ``rep_pos``:
    ``x[rep_col] = Re(r[rep_pos] * rep_scale)`` and, for paired orbits,
    ``x[rep_col + 1] = Im(r[rep_pos])`` (``symmetry.py:87-106``).
    """

    partner: np.ndarray
    phase: np.ndarray
    real_size: int
    idx_a: np.ndarray
    idx_b: np.ndarray
    coef_a: np.ndarray
    coef_b: np.ndarray
    rep_pos: np.ndarray      # independent representatives (ascending)
    rep_col: np.ndarray      # first real column of each representative
    rep_pair: np.ndarray     # 1 if the orbit has two real variables
    rep_scale: np.ndarray    # complex factor applied before taking the real part


def _self_scales(eta: np.ndarray) -> np.ndarray:
    unit = eta / np.abs(eta)
    s = np.sqrt(unit.astype(np.complex128))
    flip = np.abs(s - eta * np.conj(s)) > np.abs(-s - eta * np.conj(-s))
    return np.where(flip, -s, s)


def tilde_layout(coords: Coordinates, mode_partner: np.ndarray, mode_phase: np.ndarray) -> TildeLayout:
    """Induce the amplitude tilde map from the mode map (cc/symmetry.py:150-187)."""
    modes = coords.modes
    valid = modes >= 0
    partner_modes = np.where(valid, np.asarray(mode_partner)[np.where(valid, modes, 0)], -1)
    d = modes.shape[1]
    inv = np.zeros(modes.shape[0], np.int64)
    for i in range(d):
        for j in range(i + 1, d):
            inv += (valid[:, i] & valid[:, j] & (partner_modes[:, i] > partner_modes[:, j])).astype(np.int64)
    phase = np.prod(np.where(valid, np.asarray(mode_phase)[np.where(valid, modes, 0)], 1.0 + 0j), axis=1)
    phase = np.where(inv % 2 == 1, -phase, phase)
    # locate the partner mask: encode ascending mode tuples as integers
    base = 4 * coords.n + 1
    def encode(m):
        code = np.zeros(m.shape[0], np.int64)
        for c in range(m.shape[1]):
            code = code * base + (m[:, c] + 1)
        return code
    own = encode(np.where(valid, modes, -1))
    mapped_sorted = np.sort(np.where(valid, partner_modes, np.iinfo(np.int64).max), axis=1)
    mapped_sorted = np.where(mapped_sorted == np.iinfo(np.int64).max, -1, mapped_sorted)
    # keep -1 padding at the end for shorter tuples, like the original tuples
    tgt = encode(mapped_sorted)
    order = np.argsort(own)
    loc = np.searchsorted(own[order], tgt)
    if np.any(loc >= own.size) or np.any(own[order][np.minimum(loc, own.size - 1)] != tgt):
        raise ValueError("the coordinate set is not closed under tilde")
    partner = order[loc]
    D = coords.dimension
    idx = np.arange(D)
    rep = idx <= partner
    rep_pos = idx[rep]
    rep_pair = (partner[rep_pos] != rep_pos).astype(np.int64)
    widths = np.where(rep_pair == 1, 2, 1)
    rep_col = np.concatenate([[0], np.cumsum(widths)[:-1]]).astype(np.int64)
    real_size = int(widths.sum())
    scales = np.ones(D, np.complex128)  # read at self-partner positions only
    self_pos = rep_pos[rep_pair == 0]
    scales[self_pos] = _self_scales(phase[self_pos])
    idx_a = np.zeros(D, np.int64)
    idx_b = np.zeros(D, np.int64)
    coef_a = np.zeros(D, np.complex128)
    coef_b = np.zeros(D, np.complex128)
    col_of = np.zeros(D, np.int64)
    col_of[rep_pos] = rep_col
    # representatives
    pair_rep = rep_pos[rep_pair == 1]
    self_rep = rep_pos[rep_pair == 0]
    idx_a[pair_rep] = col_of[pair_rep]
    idx_b[pair_rep] = col_of[pair_rep] + 1
    coef_a[pair_rep] = 1.0
    coef_b[pair_rep] = 1.0j
    # partners of paired representatives: t_j = eta_i conj(x_c + i x_{c+1})
    j = partner[pair_rep]
    idx_a[j] = col_of[pair_rep]
    idx_b[j] = col_of[pair_rep] + 1
    coef_a[j] = phase[pair_rep]
    coef_b[j] = -1.0j * phase[pair_rep]
    idx_a[self_rep] = col_of[self_rep]
    idx_b[self_rep] = col_of[self_rep]
    coef_a[self_rep] = scales[self_rep]
    coef_b[self_rep] = 0.0
    rep_scale = np.where(rep_pair == 1, 1.0 + 0j, 1.0 / scales[rep_pos])
    return TildeLayout(partner, phase, real_size, idx_a, idx_b, coef_a, coef_b,
                       rep_pos, rep_col, rep_pair, rep_scale)


# ------------------------------------------------------------ padded tables
def padded_gather(coords: Coordinates, key: Key) -> tuple[np.ndarray, np.ndarray]:
    """For each padded entry of a block: canonical vector position and sign.

    Entries with a repeated index inside a group get position -1 and sign 0.
    The tables are kept on the coordinate object: the static plan, every EOM
    plan and every source plan scatter the same amplitude blocks.
    """
    cache = coords.__dict__.setdefault("_padded_gather", {})
    got = cache.get(tuple(key))
    if got is None:
        got = cache[tuple(key)] = _padded_gather(coords, key)
        for a in got:
            a.setflags(write=False)
    return got


def _padded_gather(coords: Coordinates, key: Key) -> tuple[np.ndarray, np.ndarray]:
    n = coords.n
    d = sum(key)
    size = n ** d
    pos = -np.ones(size, np.int64)
    sgn = np.zeros(size, np.int8)
    if d == 0:
        p = coords.positions(key)
        pos[:] = p[0]
        sgn[:] = 1
        return pos, sgn
    b = coords.keys.index(key)
    vpos = np.flatnonzero(coords.block_of == b)
    tup = coords.tuples[vpos, :d]
    starts = np.cumsum((0,) + tuple(key))
    strides = n ** np.arange(d - 1, -1, -1)
    for perms in product(*[list(permutations(range(c))) for c in key]):
        cols = []
        odd = False
        for g, p in enumerate(perms):
            cols.extend(int(starts[g]) + q for q in p)
            inv = sum(1 for i in range(len(p)) for k in range(i + 1, len(p)) if p[i] > p[k])
            odd ^= bool(inv % 2)
        flat = (tup[:, cols] * strides[None, :]).sum(axis=1)
        pos[flat] = vpos
        sgn[flat] = -1 if odd else 1
    return pos, sgn


def amplitude_count(n: int) -> int:
    return 2 * n * n + 2 * comb(n, 2) ** 2 + n ** 4
