"""Self-contained description of one factorized CCSD problem.

A ``ProblemSpec`` carries exactly what the coupled-cluster hot path consumes
from the reference's setup layer (``src/c3l/cc/factorized.py:248-423``):

* ``n`` -- sites per particle-hole group; the 4n modes are ordered
  (up+, up-, down+, down-) as in ``src/c3l/ci/sectors.py:23-36``;
* the distinct linear mode operators of the products, each split into a
  creator vector and an annihilator vector over the 4n modes
  (``src/c3l/cc/component_tensor.py:571-583``);
* the factorized products: coefficient and written (left-to-right) factor
  order (``src/c3l/ci/matrix_free.py:77-92``); they are applied right to left;
* the reference rapidities (one per mode);
* the mode-level tilde partners and phases (``src/c3l/ci/tilde.py:211-251``)
  from which the amplitude tilde map is induced (``src/c3l/cc/symmetry.py:150-187``);
* for every site and spin, the factor indices of the physical operators
  c, c^dagger, tilde c and tilde c^dagger used as EOM sources and sinks;
* optionally the physical one-body model (E, gamma_loss, gamma_gain of one
  spin block and the interaction sites, ``src/c3l/models.py:175-290``), which
  the Matsubara self-energy and Dyson steps read.

Specs are plain ``.npz`` files.  ``from_reference`` builds one from the
reference's ``ComponentStaticProblem`` when that package is importable.
"""

from __future__ import annotations

from dataclasses import dataclass
from pathlib import Path

import numpy as np


@dataclass(frozen=True)
class ProblemSpec:
    n: int
    creators: np.ndarray          # complex [F, 4n]
    annihilators: np.ndarray      # complex [F, 4n]
    product_coefficients: np.ndarray  # complex [P]
    product_factors: np.ndarray   # int [P, maxlen], -1 padded, written order
    product_lengths: np.ndarray   # int [P]
    rapidities: np.ndarray        # complex [4n]
    mode_partner: np.ndarray      # int [4n]
    mode_phase: np.ndarray        # complex [4n]
    source_factor: np.ndarray     # int [n, 2, 4]: c, c_dagger, tilde_c, tilde_c_dagger
    impurity_site: int = 0
    recipe: str = ""
    model_E: np.ndarray | None = None           # complex [n, n]
    model_gamma_loss: np.ndarray | None = None  # complex [n, n]
    model_gamma_gain: np.ndarray | None = None  # complex [n, n]
    interaction_sites: np.ndarray | None = None  # int [k], the impurity site first
    has_interactions: bool = True

    def __post_init__(self) -> None:
        n = int(self.n)
        M = 4 * n
        if n < 1:
            raise ValueError("n must be positive")
        for name in ("creators", "annihilators"):
            arr = np.asarray(getattr(self, name))
            if arr.ndim != 2 or arr.shape[1] != M or not np.all(np.isfinite(arr)):
                raise ValueError(f"{name} must be a finite [F, 4n] array")
        if np.asarray(self.creators).shape != np.asarray(self.annihilators).shape:
            raise ValueError("creator and annihilator tables disagree")
        if np.asarray(self.rapidities).shape != (M,):
            raise ValueError("rapidities must have one entry per mode")
        partner = np.asarray(self.mode_partner)
        if partner.shape != (M,) or not np.array_equal(partner[partner], np.arange(M)):
            raise ValueError("mode tilde partners must be an involution over the modes")
        F = np.asarray(self.creators).shape[0]
        pf = np.asarray(self.product_factors)
        pl = np.asarray(self.product_lengths)
        if pf.ndim != 2 or pl.shape != (pf.shape[0],) or np.asarray(self.product_coefficients).shape != (pf.shape[0],):
            raise ValueError("product tables are inconsistent")
        for row, ln in zip(pf, pl):
            if ln < 1 or np.any(row[:ln] < 0) or np.any(row[:ln] >= F):
                raise ValueError("a product references a missing factor")
        model = [self.model_E, self.model_gamma_loss, self.model_gamma_gain]
        if any(m is not None for m in model):
            if any(m is None or np.asarray(m).shape != (n, n) or not np.all(np.isfinite(m)) for m in model):
                raise ValueError("the physical model needs finite [n, n] E, gamma_loss and gamma_gain")
            sites = np.asarray(self.interaction_sites if self.interaction_sites is not None else [], np.int64)
            if sites.ndim != 1 or sites.size == 0 or np.any(sites < 0) or np.any(sites >= n):
                raise ValueError("interaction_sites must be a nonempty vector of sites")

    @property
    def has_model(self) -> bool:
        return self.model_E is not None

    @property
    def num_factors(self) -> int:
        return int(np.asarray(self.creators).shape[0])

    def products(self):
        for coef, row, ln in zip(self.product_coefficients, self.product_factors, self.product_lengths):
            yield complex(coef), tuple(int(f) for f in row[:ln])

    # ------------------------------------------------------------------ io
    @classmethod
    def load(cls, path: str | Path) -> "ProblemSpec":
        data = np.load(path)
        return cls(
            n=int(data["n"]),
            creators=np.asarray(data["creators"], np.complex128),
            annihilators=np.asarray(data["annihilators"], np.complex128),
            product_coefficients=np.asarray(data["product_coefficients"], np.complex128),
            product_factors=np.asarray(data["product_factors"], np.int64),
            product_lengths=np.asarray(data["product_lengths"], np.int64),
            rapidities=np.asarray(data["rapidities"], np.complex128),
            mode_partner=np.asarray(data["mode_partner"], np.int64),
            mode_phase=np.asarray(data["mode_phase"], np.complex128),
            source_factor=np.asarray(data["source_factor"], np.int64),
            impurity_site=int(data["impurity_site"]) if "impurity_site" in data else 0,
            recipe=str(data["recipe"]) if "recipe" in data else "",
            **cls._model_fields(data),
        )

    @staticmethod
    def _model_fields(data) -> dict:
        if "model_E" not in data:
            return {}
        return dict(model_E=np.asarray(data["model_E"], np.complex128),
                    model_gamma_loss=np.asarray(data["model_gamma_loss"], np.complex128),
                    model_gamma_gain=np.asarray(data["model_gamma_gain"], np.complex128),
                    interaction_sites=np.asarray(data["interaction_sites"], np.int64),
                    has_interactions=bool(data["has_interactions"]))

    def as_dict(self) -> dict:
        return {
            "n": np.int64(self.n), "creators": self.creators, "annihilators": self.annihilators,
            "product_coefficients": self.product_coefficients, "product_factors": self.product_factors,
            "product_lengths": self.product_lengths, "rapidities": self.rapidities,
            "mode_partner": self.mode_partner, "mode_phase": self.mode_phase,
            "source_factor": self.source_factor, "impurity_site": np.int64(self.impurity_site),
            "recipe": np.array(self.recipe),
        } | ({} if not self.has_model else {
            "model_E": self.model_E, "model_gamma_loss": self.model_gamma_loss,
            "model_gamma_gain": self.model_gamma_gain, "interaction_sites": self.interaction_sites,
            "has_interactions": np.bool_(self.has_interactions),
        })

    def save(self, path: str | Path) -> None:
        np.savez_compressed(path, **self.as_dict())

    # ------------------------------------------------------- reference adapter
    @classmethod
    def from_reference(cls, static_problem, recipe: str = "reference") -> "ProblemSpec":
        """Lower a reference ``ComponentStaticProblem`` (needs the reference package).

        Reads ``static_problem.oracle`` (a ``FactorizedCCProblem``,
        ``src/c3l/cc/component_tensor.py:1276-1298``).
        """
        return cls.from_factorized(static_problem.oracle, recipe)

    @classmethod
    def from_factorized(cls, cc, recipe: str = "reference") -> "ProblemSpec":
        """Lower the parts of a reference ``FactorizedCCProblem`` the hot path reads.

        ``cc`` needs ``model``, ``reference``, ``products`` and ``rapidities``
        (``src/c3l/cc/factorized.py:70-110``); the cluster masks and the
        amplitude tilde map are not read, since this package derives both
        from ``n`` and the mode-level tilde map.  Factors are numbered in
        first-use order over the products (written order), then the physical
        operators of every site and spin (``src/c3l/ci/matrix_free.py:95-139``).
        """
        from c3l.ci.matrix_free import physical_mode_operator
        from c3l.ci.tilde import tilde_map_from_references

        if cc.model.symmetry != "spin":
            raise ValueError("only the spinful (up/down conserving) layout is supported")
        n = cc.model.n_sites
        M = 4 * n
        keys: dict = {}
        cre: list = []
        ann: list = []

        def index(op) -> int:
            key = op.components
            if key not in keys:
                c = np.zeros(M, complex)
                a = np.zeros(M, complex)
                for kind, mode, coefficient in key:
                    (c if kind == "create" else a)[mode] += coefficient
                keys[key] = len(cre)
                cre.append(c)
                ann.append(a)
            return keys[key]

        maxlen = max(len(p.factors) for p in cc.products)
        pf = -np.ones((len(cc.products), maxlen), np.int64)
        pl = np.zeros(len(cc.products), np.int64)
        pc = np.zeros(len(cc.products), complex)
        for i, p in enumerate(cc.products):
            pc[i] = p.coefficient
            pl[i] = len(p.factors)
            for j, f in enumerate(p.factors):
                pf[i, j] = index(f)
        src = -np.ones((n, 2, 4), np.int64)
        for site in range(n):
            for spin in range(2):
                for k, ch in enumerate(("c", "c_dagger", "tilde_c", "tilde_c_dagger")):
                    src[site, spin, k] = index(physical_mode_operator(cc.reference, site, spin, ch))
        det = tilde_map_from_references(cc.reference.up, cc.reference.down)
        return cls(
            n=n, creators=np.asarray(cre), annihilators=np.asarray(ann),
            product_coefficients=pc, product_factors=pf, product_lengths=pl,
            rapidities=np.asarray(cc.rapidities, complex),
            mode_partner=np.asarray(det.partners, np.int64), mode_phase=np.asarray(det.factors, complex),
            source_factor=src, impurity_site=int(cc.model.impurity_site), recipe=recipe,
            **model_fields(cc.model),
        )


def model_fields(model) -> dict:
    """The one-body model of a reference ``FermionicLindbladModel`` (spin
    layout: one spin block; ``src/c3l/models.py:175-290``)."""
    return dict(model_E=np.asarray(model.E, np.complex128),
                model_gamma_loss=np.asarray(model.gamma_loss, np.complex128),
                model_gamma_gain=np.asarray(model.gamma_gain, np.complex128),
                interaction_sites=np.asarray(model.interaction_sites, np.int64),
                has_interactions=bool(model.has_interactions))
