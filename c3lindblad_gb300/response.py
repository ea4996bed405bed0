"""EOM-CCSD response on the GPU: sigma operator and G^R(omega).

Drop-in counterparts of the reference's ``eom_ccsd_problem``
(``src/c3l/cc/eom.py:93-135``), ``ComponentEOMProblem`` / ``component_eom_context`` /
``component_eom_sources`` (``src/c3l/cc/component_tensor.py:2002-2056, 2234-2251,
2816-2858``), ``ComponentSigmaOperator`` (``src/c3l/cc/component_response.py:43-58``)
and ``component_retarded_green`` (``:180-245``).

``component_retarded_green`` keeps the reference's signature and result
type but replaces one restarted GMRES per frequency by one shift-invariant
CGS2 Arnoldi basis per channel (the algorithm of ``src/c3l/green/krylov.py:284-417``),
with the reduced shifted Hessenberg solves for every frequency in one launch.
Per-frequency solution vectors are reconstructed lazily on first access.
"""

from __future__ import annotations

import resource
import time
from dataclasses import dataclass

import numpy as np
import torch

from . import runtime as rt
from .krylov import DeviceVectors, arnoldi_channels, reduced_coordinates
from .static import ComponentStaticProblem, _is_reference_object


@dataclass(frozen=True)
class EOMCCSDProblem:
    cc: ComponentStaticProblem
    response_spin: int = 0

    @property
    def dimension(self) -> int:
        n = self.cc.n
        return 2 * (n + n * n * (n - 1) // 2 + n ** 3)


def eom_ccsd_problem(cc, *, response_spin: int = 0, build_next_rank_masks: bool = False) -> EOMCCSDProblem:
    if response_spin not in (0, 1):
        raise ValueError("response_spin must be zero or one")
    return EOMCCSDProblem(ComponentStaticProblem.compile(cc), response_spin)


class ComponentEOMProblem:
    """One charge block of the S13 EOM action."""

    def __init__(self, static: ComponentStaticProblem, response_spin: int, charge: int):
        if charge not in (-1, 1):
            raise ValueError("response charge must be +1 or -1")
        self.static = static
        self.response_spin = int(response_spin)
        self.charge = int(charge)
        self._plan = None

    @classmethod
    def compile(cls, problem, static, charge: int) -> "ComponentEOMProblem":
        st = ComponentStaticProblem.compile(static)
        spin = getattr(problem, "response_spin", 0)
        return cls(st, spin, charge)

    @property
    def plan(self):
        if self._plan is None:
            from .plans import EOMPlan
            self._plan = EOMPlan(self.static.plan, self.response_spin, self.charge)
        return self._plan

    @property
    def dimension(self) -> int:
        return self.plan.dimension


class ComponentEOMContext:
    """Sigma action at fixed amplitudes (device workspace prepared once)."""

    def __init__(self, problem: ComponentEOMProblem, amplitudes):
        from .device_ops import DeviceEOM
        self.problem = problem
        st = problem.static
        if isinstance(amplitudes, torch.Tensor):
            t = amplitudes.to(torch.complex128)
        else:
            arr = np.asarray(amplitudes, dtype=np.complex128)
            if arr.shape != (st.num_amplitudes,) or not np.all(np.isfinite(arr)):
                raise ValueError("component vector has the wrong shape or is nonfinite")
            t = torch.from_numpy(arr.copy())
        self.ops = DeviceEOM(problem.plan, t, st._device)
        self.amplitudes = self.ops.amplitudes


def component_eom_context(problem, amplitudes) -> ComponentEOMContext:
    if _is_reference_object(problem):
        static = ComponentStaticProblem.compile(problem.static)
        problem = ComponentEOMProblem(static, problem.oracle.response_spin, problem.charge)
    return ComponentEOMContext(problem, amplitudes)


@dataclass
class ComponentEOMSources:
    addition: np.ndarray
    removal: np.ndarray
    sink: np.ndarray
    charge: int
    site: int
    device: tuple = ()


def component_eom_sources(context: ComponentEOMContext, *, site: int | None = None) -> ComponentEOMSources:
    spec = context.problem.static.spec
    target = spec.impurity_site if site is None else site
    if isinstance(target, (bool, np.bool_)) or not isinstance(target, (int, np.integer)) or not 0 <= int(target) < spec.n:
        raise ValueError("site is outside the auxiliary model")
    add, rem, sink = context.ops.sources(int(target))
    return ComponentEOMSources(add.cpu().numpy(), rem.cpu().numpy(), sink.cpu().numpy(), context.problem.charge,
                               int(target), (add, rem, sink))


class ComponentSigmaOperator:
    """Instrumented matrix-free retained sigma action (device)."""

    def __init__(self, context):
        if _is_reference_object(context):
            ref_problem = context.problem
            static = ComponentStaticProblem.compile(ref_problem.static)
            amps = ref_problem.static.coordinates.pack(context.amplitudes)
            context = ComponentEOMContext(ComponentEOMProblem(static, ref_problem.oracle.response_spin,
                                                              ref_problem.charge), amps)
        self.context = context
        self.dimension = context.ops.N
        self.diagonal = context.problem.plan.diagonal.copy()
        self.action_calls = 0
        self.action_wall_seconds = 0.0

    def matvec_device(self, x: torch.Tensor, out: torch.Tensor) -> None:
        self.context.ops.sigma(x, out)
        self.action_calls += 1

    def matvec(self, vector) -> np.ndarray:
        started = time.perf_counter()
        arr = np.asarray(vector, dtype=np.complex128)
        if arr.shape != (self.dimension,) or not np.all(np.isfinite(arr)):
            raise ValueError("component vector has the wrong shape or is nonfinite")
        dev = self.context.ops.device
        x = torch.from_numpy(arr.copy()).to(dev)
        out = torch.empty_like(x)
        self.context.ops.sigma(x, out)
        host = out.cpu().numpy()
        self.action_calls += 1
        self.action_wall_seconds += time.perf_counter() - started
        return host


class ComponentShiftedSolution:
    """Per-frequency record; ``solution`` is reconstructed from the shared basis on demand."""

    __slots__ = ("_channel", "_index", "converged", "info", "iterations", "true_relative_residual",
                 "residual_history", "wall_seconds")

    def __init__(self, channel, index, converged, iterations, residual, history, wall):
        self._channel = channel
        self._index = index
        self.converged = converged
        self.info = 0 if converged else 1
        self.iterations = iterations
        self.true_relative_residual = residual
        self.residual_history = history
        self.wall_seconds = wall

    @property
    def solution(self) -> np.ndarray:
        return self._channel.solutions()[self._index]


class _Channel:
    def __init__(self, basis, shifts):
        self.basis = basis
        self.shifts = shifts
        self._solutions = None

    def solutions(self) -> np.ndarray:
        if self._solutions is None:
            Y = reduced_coordinates(self.basis, self.shifts)
            m = self.basis.m
            vec = DeviceVectors(self.shifts.device)
            out = torch.zeros((Y.shape[0], self.basis.V.shape[1]), dtype=torch.complex128, device=Y.device)
            for s in range(Y.shape[0]):
                vec.axpy_c(self.basis.V, m, Y[s], 1.0, out[s])
            self._solutions = out.cpu().numpy()
        return self._solutions


@dataclass(frozen=True)
class ComponentRetardedGreen:
    omega: np.ndarray
    eta: float
    addition: np.ndarray
    removal: np.ndarray
    retarded: np.ndarray
    addition_relative_residuals: np.ndarray
    removal_relative_residuals: np.ndarray
    krylov_dimensions: tuple
    component_action_calls: int
    wall_seconds: float
    peak_rss_kib: int
    _channels: tuple = ()

    def _records(self, which: int):
        ch = self._channels[which]
        res = (self.addition_relative_residuals, self.removal_relative_residuals)[which]
        b = ch.basis
        return tuple(ComponentShiftedSolution(ch, i, bool(res[i] <= max(10 * 1e-10, b.check_residuals[-1])),
                                              b.m, float(res[i]), tuple(b.check_residuals), b.wall_seconds)
                     for i in range(res.size))

    @property
    def addition_solutions(self):
        return self._records(0)

    @property
    def removal_solutions(self):
        return self._records(1)


def component_retarded_green(operator, sources, omega, eta: float, *, rtol: float = 1.0e-10, restart: int = 40,
                             maxiter: int = 200) -> ComponentRetardedGreen:
    """Addition and removal contributions to G^R(omega) (component_response.py:180-245)."""
    op = operator if isinstance(operator, ComponentSigmaOperator) else ComponentSigmaOperator(operator)
    started = time.perf_counter()
    freq = np.asarray(omega, dtype=np.float64)
    if freq.ndim != 1 or freq.size == 0 or not np.all(np.isfinite(freq)):
        raise ValueError("omega must be a finite nonempty vector")
    dev = op.context.ops.device
    N = op.dimension
    if sources.device:
        add, rem, sink = sources.device
    else:
        add, rem, sink = (torch.from_numpy(np.asarray(v, np.complex128).copy()).to(dev)
                          for v in (sources.addition, sources.removal, sources.sink))
    if add.numel() > N:
        raise ValueError("response operator is smaller than the retained source")
    if add.numel() < N:
        pad = torch.zeros(N - add.numel(), dtype=torch.complex128, device=dev)
        add, rem, sink = (torch.cat([v, pad]) for v in (add, rem, sink))
    shifts = torch.from_numpy((freq + 1j * float(eta)).astype(np.complex128)).to(dev)
    vec = DeviceVectors(dev)
    max_dim = int(min(N, restart * maxiter, 4096))
    calls0 = op.action_calls
    out = []
    channels = []
    bases = arnoldi_channels(op.context.ops, [add.contiguous(), rem.contiguous()], shifts,
                             maximum_dimension=max_dim, residual_tolerance=rtol,
                             minimum_dimension=min(16, max_dim), check_interval=8, sink=sink.contiguous())
    op.action_calls += sum(b.m for b in bases)
    for basis in bases:
        if not basis.converged:
            raise RuntimeError("a component EOM shifted solve failed to converge")
        out.append((basis.green.cpu().numpy(), basis.residual.cpu().numpy()))
        channels.append(_Channel(basis, shifts))
    (ga, ra), (gr, rr) = out
    return ComponentRetardedGreen(
        omega=freq, eta=float(eta), addition=ga, removal=gr, retarded=ga + gr,
        addition_relative_residuals=ra, removal_relative_residuals=rr,
        krylov_dimensions=tuple(ch.basis.m for ch in channels), component_action_calls=op.action_calls - calls0,
        wall_seconds=float(time.perf_counter() - started),
        peak_rss_kib=int(resource.getrusage(resource.RUSAGE_SELF).ru_maxrss), _channels=tuple(channels))
