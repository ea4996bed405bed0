"""CPU oracle for the coupled-cluster hot path (test infrastructure only).

This module restates, in plain NumPy, the reference algorithm of
``src/c3l/cc/component_tensor.py`` for the three operations the GPU path
implements: the static CCSD residual, its Jacobian-vector product and the
EOM-CCSD sigma action.  It follows the reference's evaluation strategy on
padded antisymmetric blocks (interior products, shuffle-signed wedges and
lazily applied transformed factors), so it is slow but obviously faithful.

Only ``tests/``, ``__graft_entry__.smoke()`` and the ``cpu_baseline`` leg of
``bench.py`` may import this module.  The product path never calls it.

Parity is pinned by ``tests/test_oracle_golden.py`` against golden vectors
written by ``tests/golden/make_fixtures.py``, which runs the reference itself.
"""

from __future__ import annotations

from itertools import combinations, permutations, product
from math import comb

import numpy as np

Key = tuple  # (up+, up-, down+, down-) index counts


# ------------------------------------------------------------------ algebra
def _inversions_odd(seq) -> bool:
    """Parity of a sequence's inversions (component_tensor.py:54-60)."""
    odd = False
    for i in range(len(seq)):
        for j in range(i + 1, len(seq)):
            if seq[i] > seq[j]:
                odd = not odd
    return odd


def _shuffles(lk: Key, rk: Key):
    """Axis splits of one block wedge with their signs (component_tensor.py:63-79)."""
    per_group = []
    start = 0
    for a, b in zip(lk, rk):
        axes = list(range(start, start + a + b))
        per_group.append([c for c in combinations(axes, a)])
        start += a + b
    total = start
    for choice in product(*per_group):
        left = [ax for grp in choice for ax in grp]
        taken = set(left)
        right = [ax for ax in range(total) if ax not in taken]
        yield left, right, (-1.0 if _inversions_odd(left + right) else 1.0)


def wedge_blocks(left, lk, right, rk, n):
    """One padded block of ``left ^ right`` (component_tensor.py:82-103)."""
    deg = sum(lk) + sum(rk)
    if deg == 0:
        return np.asarray(left * right, dtype=np.complex128)
    out = np.zeros((n,) * deg, dtype=np.complex128)
    for la, ra, sign in _shuffles(lk, rk):
        out += sign * np.einsum(left, la, right, ra, list(range(deg)), optimize=False)
    return out


def add_key(a: Key, b: Key) -> Key:
    return tuple(x + y for x, y in zip(a, b))


def wedge(left: dict, right: dict, n: int, max_degree: int | None = None) -> dict:
    """Antisymmetrized product of two block forms (component_tensor.py:205-223)."""
    out: dict = {}
    for lk, lv in left.items():
        for rk, rv in right.items():
            key = add_key(lk, rk)
            if any(v > n for v in key):
                continue
            if max_degree is not None and sum(key) > max_degree:
                continue
            val = wedge_blocks(lv, lk, rv, rk, n)
            out[key] = out[key] + val if key in out else val
    return out


def interior(vectors: dict, form: dict) -> dict:
    """Bilinear contraction sum_p v_p iota_p (component_tensor.py:226-246)."""
    out: dict = {}
    for key, val in form.items():
        for g, v in vectors.items():
            if key[g] == 0:
                continue
            axis = sum(key[:g])
            tgt = list(key)
            tgt[g] -= 1
            tgt = tuple(tgt)
            c = (-1.0) ** axis * np.tensordot(v, val, axes=(0, axis))
            out[tgt] = out[tgt] + c if tgt in out else np.asarray(c, dtype=np.complex128)
    return out


def _nonzero(form: dict) -> bool:
    return any(np.any(v) for v in form.values())


def _clean(form: dict) -> dict:
    return {k: v for k, v in form.items() if np.any(v)}


def homogeneous_parts(form: dict) -> list:
    """Split a form by degree (component_tensor.py:760)."""
    degs = sorted({sum(k) for k in form})
    return [{k: v for k, v in form.items() if sum(k) == d} for d in degs]


def degree(form: dict) -> int:
    return sum(next(iter(form)))


def quadratic_action(form: dict, rapidities: np.ndarray, n: int) -> dict:
    """Bare diagonal (Lambda o form) (component_tensor.py:1236-1250)."""
    out = {}
    for key, val in form.items():
        mult = np.zeros(val.shape, dtype=np.complex128)
        axis = 0
        for g, cnt in enumerate(key):
            lam = rapidities[g * n:(g + 1) * n]
            for _ in range(cnt):
                shape = [1] * val.ndim
                shape[axis] = n
                mult = mult + lam.reshape(shape)
                axis += 1
        out[key] = mult * val
    return out


def sum_forms(*forms) -> dict:
    out: dict = {}
    for f in forms:
        for k, v in f.items():
            out[k] = out[k] + v if k in out else np.array(v, dtype=np.complex128)
    return out


# -------------------------------------------------------------- coordinates
class Coordinates:
    """Canonical coefficient positions ordered as the reference orders masks.

    Static amplitudes follow ``ness_basis`` (``ci/basis.py:149-178``): sorted by
    (particle-hole rank, bit mask).  EOM coordinates follow ``response_basis``
    (``ci/basis.py:181-236``) filtered to one charge (``component_tensor.py:2023``).
    Block positions match ``ComponentCoordinates.from_masks`` (``:275-300``).
    """

    def __init__(self, n: int, masks: list):
        self.n = n
        self.dimension = len(masks)
        recs: dict = {}
        for pos, mask in enumerate(masks):
            groups = [[], [], [], []]
            for mode in range(4 * n):
                if mask >> mode & 1:
                    groups[mode // n].append(mode % n)
            key = tuple(len(g) for g in groups)
            recs.setdefault(key, []).append((pos, tuple(i for g in groups for i in g)))
        self.blocks = []
        for key in sorted(recs):
            pos = np.array([r[0] for r in recs[key]], dtype=np.int64)
            idx = np.array([r[1] for r in recs[key]], dtype=np.int64).reshape(len(pos), sum(key))
            self.blocks.append((key, pos, idx))

    def unpack(self, vector) -> dict:
        """Canonical vector -> padded antisymmetric blocks (component_tensor.py:302-325)."""
        v = np.asarray(vector, dtype=np.complex128)
        out = {}
        for key, pos, idx in self.blocks:
            arr = np.zeros((self.n,) * sum(key), dtype=np.complex128)
            vals = v[pos]
            if sum(key) == 0:
                arr[...] = vals[0]
                out[key] = arr
                continue
            starts = np.cumsum((0,) + key)
            for perms in product(*[list(permutations(range(c))) for c in key]):
                cols = []
                sign = 1.0
                for g, p in enumerate(perms):
                    cols.extend(int(starts[g]) + q for q in p)
                    if _inversions_odd(p):
                        sign = -sign
                arr[tuple(idx[:, c] for c in cols)] = sign * vals
            out[key] = arr
        return out

    def pack(self, form: dict) -> np.ndarray:
        """Read canonical coefficients out of padded blocks (component_tensor.py:327-337)."""
        out = np.zeros(self.dimension, dtype=np.complex128)
        for key, pos, idx in self.blocks:
            val = form.get(key)
            if val is None:
                continue
            if sum(key) == 0:
                out[pos] = val
            else:
                out[pos] = val[tuple(idx[:, c] for c in range(idx.shape[1]))]
        return out


def static_masks(n: int) -> list:
    """CCSD cluster masks in reference order (factorized.py:332-338, ci/basis.py:149-178)."""
    recs = []
    up_p, up_m = range(0, n), range(n, 2 * n)
    dn_p, dn_m = range(2 * n, 3 * n), range(3 * n, 4 * n)
    for rank in (1, 2):
        for a in range(rank + 1):
            b = rank - a
            if a > n or b > n:
                continue
            for c0 in combinations(up_p, a):
                for c1 in combinations(up_m, a):
                    for c2 in combinations(dn_p, b):
                        for c3 in combinations(dn_m, b):
                            recs.append((rank, sum(1 << m for m in c0 + c1 + c2 + c3)))
    recs.sort()
    return [m for _, m in recs]


def eom_masks(n: int, spin: int, charge: int) -> list:
    """S13 response masks of one spin/charge in reference order (ci/basis.py:181-236)."""
    base = (0, 2 * n)[spin]
    other = (0, 2 * n)[1 - spin]
    rp, rm = range(base, base + n), range(base + n, base + 2 * n)
    op, om = range(other, other + n), range(other + n, other + 2 * n)
    recs = []
    for rank in (0, 1):
        for a in range(rank + 1):
            b = rank - a
            if a >= n or b > n:
                continue
            npl, nmi = (a + 1, a) if charge == 1 else (a, a + 1)
            for c0 in combinations(rp, npl):
                for c1 in combinations(rm, nmi):
                    for c2 in combinations(op, b):
                        for c3 in combinations(om, b):
                            recs.append((rank, sum(1 << m for m in c0 + c1 + c2 + c3)))
    recs.sort()
    return [m for _, m in recs]


# ------------------------------------------------------------------ tilde map
class Tilde:
    """Anti-linear orbit map of the amplitudes (cc/symmetry.py:20-200)."""

    def __init__(self, masks: list, mode_partner, mode_phase):
        index = {m: i for i, m in enumerate(masks)}
        self.partner = np.empty(len(masks), dtype=np.int64)
        self.phase = np.empty(len(masks), dtype=np.complex128)
        for i, mask in enumerate(masks):
            modes = [p for p in range(len(mode_partner)) if mask >> p & 1]
            mapped = [int(mode_partner[p]) for p in modes]
            f = complex(np.prod([mode_phase[p] for p in modes]))
            if _inversions_odd(mapped):
                f = -f
            self.partner[i] = index[sum(1 << p for p in mapped)]
            self.phase[i] = f
        self.independent = [i for i, j in enumerate(self.partner) if i <= j]
        self.real_size = sum(1 if self.partner[i] == i else 2 for i in self.independent)

    def _self_scale(self, i: int) -> complex:
        eta = self.phase[i]
        s = complex(np.sqrt(eta / abs(eta)))
        if abs(s - eta * s.conjugate()) > abs(-s - eta * (-s).conjugate()):
            s = -s
        return s

    def unpack(self, x) -> np.ndarray:
        t = np.zeros(len(self.partner), dtype=np.complex128)
        c = 0
        for i in self.independent:
            j = self.partner[i]
            if i == j:
                t[i] = self._self_scale(i) * x[c]
                c += 1
            else:
                v = x[c] + 1j * x[c + 1]
                t[i] = v
                t[j] = self.phase[i] * np.conj(v)
                c += 2
        return t

    def pack(self, t) -> np.ndarray:
        x = np.empty(self.real_size)
        c = 0
        for i in self.independent:
            if self.partner[i] == i:
                x[c] = (t[i] / self._self_scale(i)).real
                c += 1
            else:
                x[c], x[c + 1] = t[i].real, t[i].imag
                c += 2
        return x


# --------------------------------------------------------------- the problem
class OracleProblem:
    """A factorized CCSD problem built from a problem-spec dictionary."""

    def __init__(self, spec: dict):
        self.n = n = int(spec["n"])
        self.rapidities = np.asarray(spec["rapidities"], dtype=np.complex128)
        cre = np.asarray(spec["creators"])
        ann = np.asarray(spec["annihilators"])
        self.factors = []
        for f in range(cre.shape[0]):
            creator = {}
            annihilator = {}
            for g in range(4):
                c = cre[f, g * n:(g + 1) * n]
                a = ann[f, g * n:(g + 1) * n]
                if np.any(c):
                    key = tuple(1 if h == g else 0 for h in range(4))
                    creator[key] = c.astype(np.complex128)
                if np.any(a):
                    annihilator[g] = a.astype(np.complex128)
            self.factors.append((creator, annihilator))
        self.products = []
        for coef, fac, ln in zip(spec["product_coefficients"], spec["product_factors"], spec["product_lengths"]):
            self.products.append((complex(coef), [int(f) for f in fac[:ln]]))
        self.masks = static_masks(n)
        self.coords = Coordinates(n, self.masks)
        self.tilde = Tilde(self.masks, spec["mode_partner"], spec["mode_phase"])
        self.spec = spec

    # ---- lazy terms: list of (coefficient, [forms ...])
    def _apply_factor(self, states, f, shifts):
        """Apply F + [F,T] to lazy terms (component_tensor.py:764-786, 2077-2113)."""
        creator, annihilator = self.factors[f]
        wedges = ([creator] if creator else []) + list(shifts)
        out = []
        for coef, forms in states:
            for w in wedges:
                out.append((coef, [w] + forms))
            if annihilator:
                prefix = 0
                for pos, form in enumerate(forms):
                    c = interior(annihilator, form)
                    if _nonzero(c):
                        out.append((coef * (-1) ** prefix, forms[:pos] + [_clean(c)] + forms[pos + 1:]))
                    prefix += degree(form)
        return out

    def _shifts(self, form):
        """iota_a T split by degree for every factor used by a product (component_tensor.py:1387-1397)."""
        used = sorted({f for _, facs in self.products for f in facs})
        return {f: [p for p in homogeneous_parts(_clean(interior(self.factors[f][1], form))) if p] for f in used}

    def _materialize(self, terms, degrees) -> dict:
        """Wedge each lazy term and keep the listed degrees (component_tensor.py:869-898)."""
        out: dict = {}
        for coef, forms in terms:
            deg = sum(degree(f) for f in forms)
            if deg not in degrees:
                continue
            val = {(0, 0, 0, 0): np.asarray(coef, dtype=np.complex128)}
            for form in forms:
                val = wedge(val, form, self.n, max_degree=deg)
            out = sum_forms(out, val)
        return out

    def interaction(self, t: dict, dt: dict | None = None, degrees=(0, 2, 4)):
        """Sum over products of the transformed product acting on the vacuum.

        With ``dt`` the tangent (product rule of component_tensor.py:797-816)
        is returned instead of the primal.
        """
        shifts = self._shifts(t)
        dshifts = self._shifts(dt) if dt is not None else None
        total: dict = {}
        for coef, facs in self.products:
            primal = [(coef, [])]
            tangent = []
            for f in reversed(facs):
                new_primal = self._apply_factor(primal, f, shifts[f])
                if dt is not None:
                    tangent = self._apply_factor(tangent, f, shifts[f])
                    tangent += [(c, [s] + forms) for c, forms in primal for s in dshifts[f]]
                primal = new_primal
            total = sum_forms(total, self._materialize(tangent if dt is not None else primal, set(degrees)))
        return total

    def residual(self, amplitudes):
        """Static residual (component_tensor.py:1822-1868): -i pack(Lambda T + V)."""
        t = self.coords.unpack(amplitudes)
        inter = self.interaction(t)
        total = sum_forms(quadratic_action(t, self.rapidities, self.n), inter)
        ref = -1j * complex(inter.get((0, 0, 0, 0), 0.0))
        return -1j * self.coords.pack(total), ref

    def jvp(self, amplitudes, direction):
        """Exact forward tangent (component_tensor.py:1871-1930)."""
        t = self.coords.unpack(amplitudes)
        dt = self.coords.unpack(direction)
        inter = self.interaction(t, dt)
        total = sum_forms(quadratic_action(dt, self.rapidities, self.n), inter)
        ref = -1j * complex(inter.get((0, 0, 0, 0), 0.0))
        return -1j * self.coords.pack(total), ref

    def real_residual(self, x):
        return self.tilde.pack(self.residual(self.tilde.unpack(x))[0])


class OracleEOM:
    """One (spin, charge) block of the S13 sigma action at fixed amplitudes."""

    def __init__(self, problem: OracleProblem, amplitudes, spin: int = 0, charge: int = 1):
        self.p = problem
        self.spin, self.charge = spin, charge
        self.coords = Coordinates(problem.n, eom_masks(problem.n, spin, charge))
        self.t = problem.coords.unpack(amplitudes)
        self.shifts = problem._shifts(self.t)
        # vacuum interaction: all degree 0/2/4 blocks (component_tensor.py:2234-2251)
        self.vacuum = problem.interaction(self.t)
        n = problem.n
        diag = np.zeros(self.coords.dimension, dtype=np.complex128)
        for key, pos, idx in self.coords.blocks:
            axis = 0
            val = np.zeros(len(pos), dtype=np.complex128)
            for g, cnt in enumerate(key):
                for _ in range(cnt):
                    val += problem.rapidities[g * n + idx[:, axis]]
                    axis += 1
            diag[pos] = val
        self.diagonal = diag  # component_response.py:28-40
        self.plan = self._compile_plan()

    @property
    def dimension(self) -> int:
        return self.coords.dimension

    # A placeholder for the response vector: ("P", degree, contraction chain)
    def _apply_factor_plan(self, states, f):
        """Transformed factor with a placeholder input (component_tensor.py:2077-2113)."""
        creator, annihilator = self.p.factors[f]
        wedges = ([creator] if creator else []) + list(self.shifts[f])
        out = []
        for coef, forms in states:
            for w in wedges:
                out.append((coef, [w] + forms))
            if not annihilator:
                continue
            prefix = 0
            for pos, form in enumerate(forms):
                if isinstance(form, tuple):
                    deg = form[1]
                    if deg > 0:
                        out.append((coef * (-1) ** prefix, forms[:pos] + [("P", deg - 1, form[2] + (f,))] + forms[pos + 1:]))
                    prefix += deg
                else:
                    c = interior(annihilator, form)
                    if _nonzero(c):
                        out.append((coef * (-1) ** prefix, forms[:pos] + [_clean(c)] + forms[pos + 1:]))
                    prefix += degree(form)
        return out

    def _compile_plan(self):
        """Group creation forms by (input degree, contraction chain) (component_tensor.py:2116-2223)."""
        grouped: dict = {}

        def accumulate(coef, forms, d):
            pos = next(i for i, f in enumerate(forms) if isinstance(f, tuple))
            ph = forms[pos]
            after = sum(degree(f) for f in forms[pos + 1:])
            coef = coef * (-1) ** (ph[1] * after)
            creation = [f for f in forms if not isinstance(f, tuple)]
            cdeg = sum(degree(f) for f in creation)
            if cdeg + ph[1] not in (1, 3):
                return
            val = {(0, 0, 0, 0): np.asarray(coef, dtype=np.complex128)}
            for f in creation:
                val = wedge(val, f, self.p.n, max_degree=cdeg)
            key = (d, ph[2], cdeg)
            grouped[key] = sum_forms(grouped.get(key, {}), val)

        for d in (1, 3):
            for coef, facs in self.p.products:
                states = [(coef, [("P", d, ())])]
                for f in reversed(facs):
                    states = self._apply_factor_plan(states, f)
                for c, forms in states:
                    accumulate(c, forms, d)
            for key, val in self.vacuum.items():
                accumulate(-1.0, [("P", d, ()), {key: val}], d)
        return [(d, chain, _clean(form)) for (d, chain, _), form in grouped.items() if _clean(form)]

    def sigma(self, vector) -> np.ndarray:
        """Retained commutator action over the precompiled plan (component_tensor.py:2254-2302)."""
        p = self.p
        x = _clean(self.coords.unpack(vector))
        parts = {degree(h): h for h in homogeneous_parts(x) if h}
        total: dict = {}
        for d, chain, creation in self.plan:
            acted = parts.get(d)
            if acted is None:
                continue
            for f in chain:
                acted = interior(p.factors[f][1], acted)
                if not _nonzero(acted):
                    break
            else:
                out = wedge(creation, _clean(acted), p.n)
                total = sum_forms(total, {k: v for k, v in out.items() if sum(k) in (1, 3)})
        total = sum_forms(quadratic_action(x, p.rapidities, p.n), total)
        return self.coords.pack(total)

    def source(self, factor: int) -> np.ndarray:
        """pack(creator + iota_a T) (component_tensor.py:2788-2798)."""
        creator, annihilator = self.p.factors[factor]
        parts = homogeneous_parts(_clean(interior(annihilator, self.t))) if annihilator else []
        return self.coords.pack(sum_forms(creator, *parts))

    def sink(self, factor: int) -> np.ndarray:
        """Annihilator entries at degree-one coordinates (component_tensor.py:2801-2813)."""
        _, annihilator = self.p.factors[factor]
        out = np.zeros(self.coords.dimension, dtype=np.complex128)
        for key, pos, idx in self.coords.blocks:
            if sum(key) != 1:
                continue
            g = next(g for g, c in enumerate(key) if c)
            if g in annihilator:
                out[pos] = annihilator[g][idx[:, 0]]
        return out

    def sources(self, site: int):
        """Addition/removal sources and sink (component_tensor.py:2816-2858)."""
        table = self.p.spec["source_factor"][site, self.spin]  # c, c_dagger, tilde_c, tilde_c_dagger
        if self.charge == 1:
            return self.source(table[1]), -1j * self.source(table[2]), self.sink(table[0])
        return -1j * self.source(table[3]), self.source(table[0]), self.sink(table[1])


def dense_matrix(eom: OracleEOM) -> np.ndarray:
    """Explicit EOM matrix column by column (small dimensions only)."""
    d = eom.dimension
    out = np.empty((d, d), dtype=np.complex128)
    for j in range(d):
        e = np.zeros(d, dtype=np.complex128)
        e[j] = 1.0
        out[:, j] = eom.sigma(e)
    return out


def retarded_green_dense(eom: OracleEOM, site: int, omega, eta: float):
    """G^R by dense shifted solves (the quantity of component_response.py:180-245)."""
    A = dense_matrix(eom)
    add, rem, sink = eom.sources(site)
    I = np.eye(eom.dimension)
    ga = np.empty(len(omega), dtype=np.complex128)
    gr = np.empty(len(omega), dtype=np.complex128)
    for k, w in enumerate(omega):
        z = complex(w, eta)
        ga[k] = sink @ np.linalg.solve(z * I - A, add)
        gr[k] = sink @ np.linalg.solve(z * I - A, rem)
    return ga, gr, ga + gr


def amplitude_count(n: int) -> int:
    return 2 * n * n + 2 * comb(n, 2) ** 2 + n ** 4


def matrix_green_dense(eom: OracleEOM, sites, shifts):
    """G_ab(z) = sink_a . (z - K)^{-1} source_b for the addition and removal
    channels at complex shifts, by dense solves (the quantity of
    component_response.py:248-353 and 449-493).  Returns (addition, removal),
    each [len(shifts), len(sites), len(sites)] with axes (z, sink, source)."""
    A = dense_matrix(eom)
    I = np.eye(eom.dimension)
    cols = [eom.sources(s) for s in sites]
    sinks = np.vstack([c[2] for c in cols])
    add = np.vstack([c[0] for c in cols]).T
    rem = np.vstack([c[1] for c in cols]).T
    z = np.asarray(shifts, dtype=np.complex128)
    S = len(cols)
    rhs = np.hstack([add, rem])
    ga = np.empty((z.size, S, S), dtype=np.complex128)
    gr = np.empty_like(ga)
    for k, zk in enumerate(z):
        g = sinks @ np.linalg.solve(zk * I - A, rhs)  # one factorization for both channels
        ga[k], gr[k] = g[:, :S], g[:, S:]
    return ga, gr


def matrix_time_dense(eom: OracleEOM, sites, times):
    """-i sink_a . exp(-i K t) source_b for the combined (addition + removal),
    addition and removal sources (the quantity of component_response.py:628-663
    and 685-815), by dense matrix exponentials.  Each result is
    [len(times), len(sites), len(sites)]."""
    from scipy.linalg import expm

    A = dense_matrix(eom)
    cols = [eom.sources(s) for s in sites]
    sinks = np.vstack([c[2] for c in cols])
    add = np.vstack([c[0] for c in cols]).T
    rem = np.vstack([c[1] for c in cols]).T
    t = np.asarray(times, dtype=np.float64)
    out = [np.empty((t.size, len(cols), len(cols)), dtype=np.complex128) for _ in range(3)]
    for k, tk in enumerate(t):
        P = expm(-1j * tk * A)
        pa, pr = P @ add, P @ rem
        out[1][k] = -1j * (sinks @ pa)
        out[2][k] = -1j * (sinks @ pr)
        out[0][k] = out[1][k] + out[2][k]
    return tuple(out)
