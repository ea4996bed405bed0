"""Device plans for the static residual/JVP and the EOM sigma action.

A plan bundles the compiled program (``compiler.Program``) with the index
tables that move data between the reference's vector layouts and the padded
workspace blocks: tilde unpacking, canonical -> padded scatter, and the
per-output epilogue data (rapidity sums, real-coordinate columns).
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .compiler import Atom, Builder, Symbolic, compile_output, eom_terms, static_terms
from .layout import Coordinates, eom_coordinates, padded_gather, static_coordinates, tilde_layout
from .spec import ProblemSpec


@dataclass
class ScatterTable:
    """Canonical vector -> padded blocks: ``ws[off + e] = sign[e] * vec[pos[e]]``."""

    dst: np.ndarray   # int64 workspace offsets
    pos: np.ndarray   # int64 source positions (0 where sign == 0)
    sign: np.ndarray  # float64 (+1, -1, 0)


def _scatter_table(coords: Coordinates, offsets: dict) -> ScatterTable:
    dst, pos, sgn = [], [], []
    for key, off in offsets.items():
        p, s = padded_gather(coords, key)
        dst.append(off + np.arange(p.size, dtype=np.int64))
        pos.append(np.where(p >= 0, p, 0))
        sgn.append(s.astype(np.float64))
    return ScatterTable(np.concatenate(dst), np.concatenate(pos), np.concatenate(sgn))


class StaticPlan:
    """Residual and exact JVP of one factorized CCSD problem.

    Mirrors ``component_static_residual`` / ``component_static_linearization``
    / ``component_static_linearized_jvp`` (``src/c3l/cc/component_tensor.py:1371-1868``)
    in the real tilde coordinates of ``src/c3l/cc/component_solver.py:57-74``.
    """

    def __init__(self, spec: ProblemSpec):
        self.spec = spec
        self.n = n = spec.n
        self.coords = coords = static_coordinates(n)
        self.tilde = tilde_layout(coords, spec.mode_partner, spec.mode_phase)
        self.sym = sym = Symbolic(spec, coords)
        self.res_terms, self.jvp_terms = static_terms(sym, spec)
        b = Builder(sym, spec)
        b.add_source("T", coords.keys)
        b.add_source("V", coords.keys)
        rep = self.tilde.rep_pos
        allpos = np.arange(coords.dimension)
        # real-coordinate outputs at tilde representatives (Newton path) and
        # complex outputs -i(...) at every coordinate (arbitrary amplitudes)
        self.res_scalar_off = compile_output(b, "res", self.res_terms, coords, rep, "res_rest", "res_scalar",
                                             extra=(("res_all", allpos, -1j),), pairs=True)
        # the inner JVP of the mixed solve reads its outputs through pair GEMMs
        self.jvp_scalar_off = compile_output(b, "jvp", self.jvp_terms, coords, rep, "jvp_rest", "jvp_scalar",
                                             extra=(("jvp_all", allpos, -1j),), pairs=True)
        self.program = b.finish()
        self.scatter_T = _scatter_table(coords, self.program.source_offsets["T"])
        self.scatter_V = _scatter_table(coords, self.program.source_offsets["V"])
        lam = coords.rapidity_sum(spec.rapidities)
        self.rapidity_diagonal = -1j * lam          # newton_krylov.py:137-155
        self.lam_all = -1j * lam[self.program.stages["res_all"].elements]
        self.lam_all_jvp = -1j * lam[self.program.stages["jvp_all"].elements]
        # epilogue per canonical output element (elements are tilde representatives)
        out = self.program.stages["res"]
        self.epilogue = self._epilogue(out.elements, lam)
        self.epilogue_jvp = self._epilogue(self.program.stages["jvp"].elements, lam)

    def _epilogue(self, elements: np.ndarray, lam: np.ndarray) -> dict:
        t = self.tilde
        col_of = np.zeros(self.coords.dimension, np.int64)
        col_of[t.rep_pos] = t.rep_col
        pair_of = np.zeros(self.coords.dimension, np.int64)
        pair_of[t.rep_pos] = t.rep_pair
        scale_of = np.ones(self.coords.dimension, np.complex128)
        scale_of[t.rep_pos] = t.rep_scale
        return dict(lam=lam[elements], col=col_of[elements], pair=pair_of[elements], scale=scale_of[elements])

    @property
    def num_amplitudes(self) -> int:
        return self.coords.dimension

    @property
    def num_variables(self) -> int:
        return self.tilde.real_size

    def preconditioner_table(self):
        """Real 2x2 (or 1x1) blocks of ``pack(unpack(x) / diag)`` (newton_krylov.py:158-192)."""
        diag = np.array(self.rapidity_diagonal, copy=True)
        mag = np.abs(diag)
        scale = max(float(np.max(mag, initial=0.0)), 1.0)
        thr = 1.0e-12 * scale
        small = mag < thr
        if np.any(small):
            diag[small] = thr * np.exp(1j * np.angle(diag[small] + 1.0e-300))
        t = self.tilde
        inv = 1.0 / diag[t.rep_pos]
        # pair: (a + ib) * inv -> [Re, Im]; self: Re(s x inv / s) = Re(inv) x
        m = np.zeros((t.rep_pos.size, 4), np.float64)
        m[:, 0] = inv.real
        m[:, 1] = -inv.imag
        m[:, 2] = inv.imag
        m[:, 3] = inv.real
        finite = mag[~small]
        diagnostics = dict(
            minimum_magnitude=float(np.min(finite)) if finite.size else thr,
            maximum_magnitude=float(np.max(mag, initial=thr)),
            regularization_threshold=thr, regularized_amplitudes=int(np.count_nonzero(small)),
        )
        diagnostics["magnitude_condition"] = diagnostics["maximum_magnitude"] / max(diagnostics["minimum_magnitude"], thr)
        return m, diagnostics


class EOMPlan:
    """S13 sigma action of one (spin, charge) block, or with ``space="S135"``
    the full action among S1, S3 and the rank-five shell S5.

    Mirrors ``component_eom_context`` / ``component_eom_sigma``
    (``src/c3l/cc/component_tensor.py:2234-2302``) and ``FullS135ResponseOperator``
    (``src/c3l/cc/s135_full.py:296-361``).
    """

    def __init__(self, static: StaticPlan, spin: int = 0, charge: int = 1, space: str = "S13"):
        if spin not in (0, 1) or charge not in (1, -1):
            raise ValueError("response spin must be 0/1 and charge +1/-1")
        spec = static.spec
        self.static = static
        self.spin, self.charge, self.space = spin, charge, space
        n = spec.n
        if space == "S135" and n ** 5 >= 2 ** 31:
            raise ValueError("the rank-five padded blocks need n**5 < 2**31 (n <= 73)")
        self.coords = coords = eom_coordinates(n, spin, charge, space)
        sym = Symbolic(spec, static.coords, coords.keys)
        self.sym = sym
        # the vacuum interaction uses the static monomials (all degree 0/2/4 blocks)
        self.sigma_terms = eom_terms(sym, spec, coords.keys, static.res_terms)
        b = Builder(sym, spec)
        b.add_source("T", static.coords.keys)
        b.add_source("X", coords.keys)
        allpos = np.arange(coords.dimension)
        # the output stage sums its anchor ^ rest products as pair GEMMs
        compile_output(b, "sigma", self.sigma_terms, coords, allpos, "sigma_rest", None, pairs=True)
        self.program = b.finish()
        self.scatter_T = _scatter_table(static.coords, self.program.source_offsets["T"])
        self.scatter_X = _scatter_table(coords, self.program.source_offsets["X"])
        lam = coords.rapidity_sum(spec.rapidities)
        self.diagonal = lam                                   # component_response.py:28-40
        self.lam_sigma = lam[self.program.stages["sigma"].elements]
        self._sources: dict = {}

    @property
    def dimension(self) -> int:
        return self.coords.dimension

    def sources(self, site: int) -> "SourcePlan":
        got = self._sources.get(site)
        if got is None:
            got = SourcePlan(self, site)
            self._sources[site] = got
        return got


class SourcePlan:
    """Addition/removal sources and the trace sink of one site.

    Sources are ``pack(creator + iota_a T)`` of a physical operator, scaled
    by ``-i`` for the tilde channel; the sink is the annihilator part at
    degree-one coordinates (``src/c3l/cc/component_tensor.py:2788-2858``).
    """

    def __init__(self, eom: EOMPlan, site: int):
        spec = eom.static.spec
        n = spec.n
        if not 0 <= int(site) < n:
            raise ValueError("site is outside the auxiliary model")
        self.site = int(site)
        coords = eom.coords
        table = spec.source_factor[self.site, eom.spin]  # c, c_dagger, tilde_c, tilde_c_dagger
        if eom.charge == 1:
            add_f, rem_f, sink_f = int(table[1]), int(table[2]), int(table[0])
            self.source_scale = (1.0 + 0j, -1j)
        else:
            add_f, rem_f, sink_f = int(table[3]), int(table[0]), int(table[1])
            self.source_scale = (-1j, 1.0 + 0j)
        sym = Symbolic(spec, eom.static.coords, coords.keys)
        b = Builder(sym, spec)
        b.add_source("T", eom.static.coords.keys)
        allpos = np.arange(coords.dimension)
        for name, f in (("add", add_f), ("rem", rem_f)):
            terms = {}
            for part in (1, 3):
                a = Atom("T", f, part)
                if sym.nonzero(a):
                    terms[(a,)] = 1.0 + 0j
            compile_output(b, name, terms, coords, allpos, f"{name}_rest", None)
        self.program = b.finish()
        self.scatter_T = _scatter_table(eom.static.coords, self.program.source_offsets["T"])
        ann = np.asarray(spec.annihilators[sink_f])
        sink = np.zeros(coords.dimension, np.complex128)
        for b_id, key in enumerate(coords.keys):
            if sum(key) != 1:
                continue
            g = key.index(1)
            p = np.flatnonzero(coords.block_of == b_id)
            sink[p] = ann[g * n + coords.tuples[p, 0]]
        self.sink = sink
