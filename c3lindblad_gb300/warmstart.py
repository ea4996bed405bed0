"""Learned warm start for the static CCSD solve.

An element-wise MLP corrects the first-order guess ``t1 = -M^-1 r(0)`` (one
preconditioned Jacobi step from zero amplitudes, M the rapidity diagonal of
``src/c3l/cc/newton_krylov.py:137-192``).  Per tilde-orbit representative it
sees the rapidities of the amplitude's modes (orbital energies and loss/gain
rates in the normal-mode basis), a singles/doubles flag, the interaction
scale U, t1 and the second Jacobi iterate ``t2 = t1 - M^-1 r(t1)``, and
predicts ``(x* - t1) / sigma`` with sigma the RMS of t1.  It is trained on the amplitudes this package's own GPU solver
converges to on seeded models, with the library's BF16 forward/backward and
Adam kernels.  The zero guess stays the fallback: the solver keeps the
learned guess only if its FP64 residual is smaller, and convergence of the
FP64 residual judges the answer either way.
"""

from __future__ import annotations

import time
from dataclasses import dataclass
from pathlib import Path

import numpy as np
import torch

from . import runtime as rt

F, H, O = 16, 32, 2
PARAMS = H * F + H + H * H + H + O * H + O


def init_params(seed: int = 0) -> np.ndarray:
    """Glorot-scaled weights, zero biases (layout W1 b1 W2 b2 W3 b3)."""
    rng = np.random.default_rng(seed)
    parts = [rng.normal(0, np.sqrt(1.0 / F), H * F), np.zeros(H),
             rng.normal(0, np.sqrt(1.0 / H), H * H), np.zeros(H),
             rng.normal(0, 0.1 * np.sqrt(1.0 / H), O * H), np.zeros(O)]
    return np.concatenate(parts).astype(np.float32)


def interaction_scale(spec) -> float:
    """Mean |coefficient| of the products with four or more factors (0 if none)."""
    coefs = [abs(c) for c, facs in spec.products() if len(facs) >= 4]
    return float(np.mean(coefs)) if coefs else 0.0


class MLPDevice:
    """FP32 master parameters, their BF16 copy and Adam state on one device."""

    def __init__(self, params: np.ndarray, device):
        if params.shape != (PARAMS,):
            raise ValueError("parameter vector has the wrong size")
        self.device = device
        self.lib = rt.lib()
        self.p = torch.from_numpy(np.asarray(params, np.float32).copy()).to(device)
        self.pb = self.p.to(torch.bfloat16)
        self.m = torch.zeros_like(self.p)
        self.v = torch.zeros_like(self.p)
        self.g = torch.zeros_like(self.p)
        self.loss = torch.zeros(1, dtype=torch.float32, device=device)
        self.steps = 0

    def s(self) -> int:
        return rt.stream_ptr(self.device)

    def forward(self, X: torch.Tensor) -> torch.Tensor:
        n = X.shape[0]
        Y = torch.empty((n, O), dtype=torch.float32, device=self.device)
        rt.check(self.lib.c3l_mlp_forward(n, X.data_ptr(), self.pb.data_ptr(), Y.data_ptr(), self.s()), "mlp forward")
        rt.LaunchCounter.add(1)
        return Y

    def gradient(self, X: torch.Tensor, T: torch.Tensor, W: torch.Tensor | None = None, wsum: float | None = None):
        n = X.shape[0]
        self.g.zero_()
        self.loss.zero_()
        inv = 1.0 / (float(n) if wsum is None else wsum)
        rt.check(self.lib.c3l_mlp_backward(n, X.data_ptr(), T.data_ptr(), rt.ptr(W), inv, self.pb.data_ptr(),
                                           self.g.data_ptr(), self.loss.data_ptr(), self.s()), "mlp backward")
        rt.LaunchCounter.add(1)
        return self.g, self.loss

    def adam(self, lr: float, beta1: float = 0.9, beta2: float = 0.999, eps: float = 1e-8) -> None:
        self.steps += 1
        rt.check(self.lib.c3l_mlp_adam(self.p.data_ptr(), self.g.data_ptr(), self.m.data_ptr(), self.v.data_ptr(),
                                       lr, beta1, beta2, eps, self.steps, self.pb.data_ptr(), self.s()), "adam")
        rt.LaunchCounter.add(1)

    def params(self) -> np.ndarray:
        return self.p.cpu().numpy().copy()


def _rep_modes(plan) -> np.ndarray:
    modes = plan.coords.modes[plan.tilde.rep_pos]
    out = -np.ones((modes.shape[0], 4), np.int64)
    out[:, :modes.shape[1]] = modes
    return out


class _ProblemFeatures:
    """Device tables of one problem needed to build features and guesses."""

    def __init__(self, problem):
        ops = problem.ops
        plan = problem.plan
        dev = ops.device
        self.ops = ops
        self.nrep = int(plan.tilde.rep_pos.size)
        self.modes = torch.from_numpy(_rep_modes(plan)).to(dev)
        self.col = ops.pc_col
        self.pair = ops.pc_pair
        self.rap = torch.from_numpy(np.asarray(problem.spec.rapidities, np.complex128)).to(dev)
        self.u = interaction_scale(problem.spec)

    def first_order(self):
        """Jacobi iterates t1 = -M^-1 r(0), t2 = t1 - M^-1 r(t1) and sigma = RMS(t1)."""
        from .krylov import DeviceVectors

        ops = self.ops
        dev = ops.device
        vec = DeviceVectors(dev)
        zero = torch.zeros(ops.D, dtype=torch.float64, device=dev)
        r = torch.empty_like(zero)
        ops.residual(zero, r)
        t1 = torch.empty_like(zero)
        ops.precondition(r, t1)
        vec.scale_r(-1.0, t1, t1)
        ops.residual(t1, r)
        step = torch.empty_like(zero)
        ops.precondition(r, step)
        t2 = t1.clone()
        vec.axpy_r(step, 1, vec.one_r, -1.0, t2)
        sigma = max(vec.norm_r(t1) / np.sqrt(ops.D), 1e-300)
        self.t2 = t2
        return t1, sigma

    def features(self, t1: torch.Tensor, sigma: float) -> torch.Tensor:
        X = torch.empty((self.nrep, F), dtype=torch.bfloat16, device=t1.device)
        rt.check(rt.lib().c3l_warm_features(self.nrep, self.modes.data_ptr(), self.col.data_ptr(), self.pair.data_ptr(),
                                            self.rap.data_ptr(), t1.data_ptr(), self.t2.data_ptr(), float(sigma),
                                            float(self.u), X.data_ptr(), rt.stream_ptr(t1.device)), "warm features")
        rt.LaunchCounter.add(1)
        return X

    def targets(self, xstar: np.ndarray, t1: torch.Tensor, sigma: float) -> torch.Tensor:
        t1h = t1.cpu().numpy()
        col = self.col.cpu().numpy()
        pair = self.pair.cpu().numpy()
        T = np.zeros((self.nrep, O), np.float32)
        T[:, 0] = (xstar[col] - t1h[col]) / sigma
        pr = pair == 1
        T[pr, 1] = (xstar[col[pr] + 1] - t1h[col[pr] + 1]) / sigma
        return torch.from_numpy(T).to(t1.device)


class LearnedWarmStart:
    """Initial real tilde coordinates from the trained network (see module docstring)."""

    label = "learned"

    def __init__(self, params: np.ndarray, meta: dict | None = None):
        self.params = np.asarray(params, np.float32)
        if self.params.shape != (PARAMS,):
            raise ValueError("parameter vector has the wrong size")
        self.meta = dict(meta or {})
        self._dev: dict = {}

    def save(self, path) -> None:
        np.savez_compressed(path, params=self.params, **{k: np.asarray(v) for k, v in self.meta.items()})

    @classmethod
    def load(cls, path) -> "LearnedWarmStart":
        data = np.load(path)
        meta = {k: data[k] for k in data.files if k != "params"}
        return cls(data["params"], meta)

    def _mlp(self, device) -> MLPDevice:
        key = str(device)
        if key not in self._dev:
            self._dev[key] = MLPDevice(self.params, device)
        return self._dev[key]

    def initial_variables(self, problem) -> torch.Tensor:
        feats = problem.__dict__.get("_warm_features")
        if feats is None:
            feats = _ProblemFeatures(problem)
            problem.__dict__["_warm_features"] = feats
        t1, sigma = feats.first_order()
        X = feats.features(t1, sigma)
        Y = self._mlp(t1.device).forward(X)
        x0 = t1.clone()
        rt.check(rt.lib().c3l_warm_apply(feats.nrep, feats.col.data_ptr(), feats.pair.data_ptr(), t1.data_ptr(),
                                         Y.data_ptr(), float(sigma), x0.data_ptr(), rt.stream_ptr(t1.device)),
                 "warm apply")
        rt.LaunchCounter.add(1)
        return self.safeguard(problem, x0)

    @staticmethod
    def safeguard(problem, x0: torch.Tensor, scales=(1.0, 0.5, 0.25, 0.125)) -> torch.Tensor:
        """Backtrack along the guess: keep the scaled guess with the lowest FP64
        residual, or the zero guess if none beats it."""
        from .krylov import DeviceVectors

        ops = problem.ops
        vec = DeviceVectors(x0.device)
        r = torch.empty_like(x0)
        ops.residual(torch.zeros_like(x0), r)
        best, best_norm = torch.zeros_like(x0), vec.norm_r(r)
        trial = torch.empty_like(x0)
        for a in scales:
            vec.scale_r(a, x0, trial)
            ops.residual(trial, r)
            nrm = vec.norm_r(r)
            if nrm < best_norm:
                best_norm = nrm
                best = trial.clone()
        return best


@dataclass
class TrainingReport:
    models: int
    samples: int
    epochs: int
    initial_loss: float
    final_loss: float
    collect_seconds: float
    train_seconds: float


def collect(problems, *, precision: str = "mixed"):
    """Features and targets from this package's own converged solutions."""
    from .static import solve_component_ccsd

    Xs, Ts = [], []
    for p in problems:
        sol = solve_component_ccsd(p, precision=precision)
        if not sol.converged:
            continue
        feats = _ProblemFeatures(p)
        p.__dict__["_warm_features"] = feats
        t1, sigma = feats.first_order()
        Xs.append(feats.features(t1, sigma))
        Ts.append(feats.targets(sol.variables, t1, sigma))
    return torch.cat(Xs), torch.cat(Ts)


def train(X: torch.Tensor, T: torch.Tensor, *, epochs: int = 400, lr: float = 3e-3, seed: int = 0,
          init: np.ndarray | None = None) -> tuple[LearnedWarmStart, list]:
    """Full-batch Adam on the device; returns the network and the loss history."""
    mlp = MLPDevice(init_params(seed) if init is None else init, X.device)
    n = X.shape[0]
    history = []
    for epoch in range(epochs):
        _, loss = mlp.gradient(X, T)
        mlp.adam(lr)
        if epoch % 50 == 0 or epoch == epochs - 1:
            history.append(float(loss.item()) / n)
    return LearnedWarmStart(mlp.params()), history


def load_family(path, device=None):
    """Problems of a model family file written by ``tests/golden/make_fixtures.py warmstart``."""
    from .spec import ProblemSpec
    from .static import ComponentStaticProblem

    data = np.load(path)
    out = []
    for i in range(int(data["count"])):
        kw = {k[len(f"m{i}_"):]: data[k] for k in data.files if k.startswith(f"m{i}_")}
        spec = ProblemSpec(n=int(kw["n"]), creators=kw["creators"], annihilators=kw["annihilators"],
                           product_coefficients=kw["product_coefficients"], product_factors=kw["product_factors"],
                           product_lengths=kw["product_lengths"], rapidities=kw["rapidities"],
                           mode_partner=kw["mode_partner"], mode_phase=kw["mode_phase"],
                           source_factor=kw["source_factor"], impurity_site=int(kw["impurity_site"]),
                           recipe=str(kw["recipe"]))
        out.append(ComponentStaticProblem(spec, device=device))
    return out


def main(argv=None) -> None:
    """Train on a model family and write the network: ``python -m c3lindblad_gb300.warmstart FAMILY OUT``."""
    import argparse
    import json

    ap = argparse.ArgumentParser()
    ap.add_argument("family")
    ap.add_argument("out")
    ap.add_argument("--train", type=int, default=48)
    ap.add_argument("--epochs", type=int, default=600)
    ap.add_argument("--lr", type=float, default=3e-3)
    args = ap.parse_args(argv)
    dev = rt.require_cuda()
    problems = load_family(args.family, dev)
    t0 = time.perf_counter()
    X, T = collect(problems[:args.train])
    t1 = time.perf_counter()
    ws, hist = train(X, T, epochs=args.epochs, lr=args.lr)
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    ws.meta = {"family": Path(args.family).name, "train_models": args.train, "samples": X.shape[0],
               "epochs": args.epochs, "loss_history": np.asarray(hist)}
    ws.save(args.out)
    print(json.dumps({"samples": int(X.shape[0]), "collect_s": t1 - t0, "train_s": t2 - t1, "loss": hist}))


if __name__ == "__main__":
    main()
