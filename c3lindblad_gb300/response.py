"""EOM-CCSD response on the GPU: sigma operator and G^R(omega).

Drop-in counterparts of the reference's ``eom_ccsd_problem``
(``src/c3l/cc/eom.py:93-135``), ``ComponentEOMProblem`` / ``component_eom_context`` /
``component_eom_sources`` (``src/c3l/cc/component_tensor.py:2002-2056, 2234-2251,
2816-2858``), ``ComponentSigmaOperator`` (``src/c3l/cc/component_response.py:43-58``)
and ``component_retarded_green`` (``:180-245``).

``component_retarded_green`` keeps the reference's signature and result
type but replaces one restarted GMRES per frequency by one shift-invariant
CGS2 Arnoldi basis per channel (the algorithm of ``src/c3l/green/krylov.py:284-417``),
with the reduced shifted Hessenberg solves for every frequency advanced on the
device as the basis grows.  Per-frequency solution vectors are reconstructed
lazily on first access.  ``component_retarded_matrix_green_arnoldi`` is the
many-source form (``src/c3l/cc/component_response.py:356-423, 550-625``): all
addition/removal channels of all sources run as concurrent Arnoldi channels,
and every sink row is contracted from each channel's basis.
"""

from __future__ import annotations

import ctypes as C
import dataclasses
import resource
import time
from dataclasses import dataclass
from time import perf_counter

import numpy as np
import torch

from . import runtime as rt
from .krylov import DeviceVectors, arnoldi_channels, hessenberg_coordinates, reduced_coordinates
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
    """One charge block of the S13 EOM action (``space="S135"``: the full
    action on S1 + S3 + the rank-five shell, used by ``FullS135ResponseOperator``)."""

    def __init__(self, static: ComponentStaticProblem, response_spin: int, charge: int, *, space: str = "S13"):
        if charge not in (-1, 1):
            raise ValueError("response charge must be +1 or -1")
        if space not in ("S13", "S135"):
            raise ValueError("space must be 'S13' or 'S135'")
        self.static = static
        self.response_spin = int(response_spin)
        self.charge = int(charge)
        self.space = space
        self._plan = None
        self._tables = {}  # device -> Uploader holding this problem's program tables (shared by contexts)

    @classmethod
    def compile(cls, problem, static, charge: int) -> "ComponentEOMProblem":
        st = ComponentStaticProblem.compile(static)
        spin = getattr(problem, "response_spin", 0)
        return cls(st, spin, charge)

    @property
    def plan(self):
        if self._plan is None:
            from .plans import EOMPlan
            self._plan = EOMPlan(self.static.plan, self.response_spin, self.charge, self.space)
        return self._plan

    @property
    def dimension(self) -> int:
        return self.plan.dimension


class ComponentEOMContext:
    """Sigma action at fixed amplitudes (device workspace prepared once)."""

    def __init__(self, problem: ComponentEOMProblem, amplitudes, *, interaction_scale: float = 1.0):
        """``interaction_scale``: the homotopy scale the amplitudes solve
        (``solve_component_ccsd(..., interaction_scale=s)``); the sigma
        action's product part is scaled by it."""
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
        self.ops = DeviceEOM(problem.plan, t, st._device, tables=problem._tables, interaction_scale=interaction_scale)
        self.amplitudes = self.ops.amplitudes
        self.interaction_scale = float(interaction_scale)


def component_eom_context(problem, amplitudes, *, interaction_scale: float = 1.0) -> ComponentEOMContext:
    if _is_reference_object(problem):
        static = ComponentStaticProblem.compile(problem.static)
        problem = ComponentEOMProblem(static, problem.oracle.response_spin, problem.charge)
    return ComponentEOMContext(problem, amplitudes, interaction_scale=interaction_scale)


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

    __slots__ = ("_channel", "_index", "_solution", "converged", "info", "iterations", "true_relative_residual",
                 "residual_history", "wall_seconds")

    def __init__(self, channel, index, converged, iterations, residual, history, wall, *, solution=None, info=None):
        self._channel = channel
        self._index = index
        self._solution = solution
        self.converged = converged
        self.info = (0 if converged else 1) if info is None else int(info)
        self.iterations = iterations
        self.true_relative_residual = residual
        self.residual_history = history
        self.wall_seconds = wall

    @property
    def solution(self) -> np.ndarray:
        if self._solution is not None or self._channel is None:
            return self._solution
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


class _ShiftedGMRES:
    """Device buffers of ``c3l_gmres_shifted`` for one operator and restart."""

    def __init__(self, ops, restart: int):
        dev = ops.device
        n = ops.N
        r = int(min(restart, n))
        lib = rt.lib()
        self.ops, self.restart = ops, r
        self.V = torch.empty((r + 1, n), dtype=torch.complex128, device=dev)
        self.tmp = torch.empty(n, dtype=torch.complex128, device=dev)
        self.r = torch.empty(n, dtype=torch.complex128, device=dev)
        self.coeff = torch.zeros(2 * (r + 2) + 4, dtype=torch.complex128, device=dev)
        self.partial = torch.empty(max(int(lib.c3l_multi_dot_scratch(r + 1, n)), 1), dtype=torch.complex128,
                                   device=dev)
        self.host = torch.zeros(3 * (r + 2) + 4, dtype=torch.complex128).pin_memory()
        self.history = np.zeros(8192, dtype=np.float64)
        self.pc = torch.empty(n, dtype=torch.complex128, device=dev)

    def solve(self, shift: complex, inverse: np.ndarray, b: torch.Tensor, x: torch.Tensor, *, rtol: float,
              maxiter: int, use_x0: bool):
        ops = self.ops
        self.pc.copy_(torch.from_numpy(inverse))
        a = rt.GmresShiftedArgs()
        a.sigma = C.addressof(ops.sigma_action)
        a.sigma_launches = int(ops.sigma_launches)
        a.use_x0 = 1 if use_x0 else 0
        a.dim = ops.N
        a.shift = rt.cplx(shift)
        a.pc_inv, a.b, a.x = self.pc.data_ptr(), b.data_ptr(), x.data_ptr()
        a.rtol, a.atol = float(rtol), 0.0
        a.restart, a.maxiter = self.restart, int(maxiter)
        a.V, a.tmp, a.r = self.V.data_ptr(), self.tmp.data_ptr(), self.r.data_ptr()
        a.coeff, a.partial, a.host = self.coeff.data_ptr(), self.partial.data_ptr(), self.host.data_ptr()
        a.history, a.history_capacity = self.history.ctypes.data, self.history.size
        rt.check(rt.lib().c3l_gmres_shifted(C.byref(a), rt.stream_ptr(ops.device)), "gmres_shifted")
        rt.LaunchCounter.add(int(a.launches))
        return int(a.info), list(self.history[:min(a.history_len, self.history.size)]), int(a.matvecs)


def _true_relative_residual(ops, shift: complex, x: torch.Tensor, b: torch.Tensor, bnorm: float) -> float:
    """|b - (z x - K x)| / |b| on the device (component_response.py:117-118)."""
    lib = rt.lib()
    kx = torch.empty_like(x)
    ops.sigma(x, kx)
    ax = torch.empty_like(x)
    rt.check(lib.c3l_shifted_combine(x.numel(), rt.cplx(shift), x.data_ptr(), kx.data_ptr(), None, ax.data_ptr(),
                                     rt.stream_ptr(ops.device)), "shifted_combine")
    rt.LaunchCounter.add(1)
    return float(torch.linalg.vector_norm(b - ax).item()) / max(bnorm, np.finfo(float).tiny)


def _jacobi_inverse(diagonal: np.ndarray, shift: complex) -> np.ndarray:
    """(z - diag)^{-1} with entries below sqrt(eps) left at 1 (component_response.py:88-93)."""
    d = shift - diagonal
    inverse = np.ones_like(d)
    safe = np.abs(d) > np.sqrt(np.finfo(np.float64).eps)
    inverse[safe] = 1.0 / d[safe]
    return inverse


def solve_component_shifted(operator, shift: complex, rhs, *, rtol: float = 1.0e-10, restart: int = 40,
                            maxiter: int = 200, initial_solution=None) -> "ComponentShiftedSolution":
    """Solve (z I - K) x = b by preconditioned restarted GMRES on the device.

    Same signature, convergence rule and record as the reference
    (``src/c3l/cc/component_response.py:72-128``): converged iff GMRES
    reports success and the true relative residual is at most
    max(10 rtol, 1e-12).
    """
    op = operator if isinstance(operator, ComponentSigmaOperator) else ComponentSigmaOperator(operator)
    b = np.asarray(rhs, dtype=np.complex128)
    if b.shape != (op.dimension,) or not np.all(np.isfinite(b)):
        raise ValueError("shifted-response source has the wrong shape or is nonfinite")
    ops = op.context.ops
    dev = ops.device
    started = time.perf_counter()
    bd = torch.from_numpy(b.copy()).to(dev)
    x = torch.zeros_like(bd)
    if initial_solution is not None:
        x.copy_(torch.from_numpy(np.asarray(initial_solution, dtype=np.complex128).copy()))
    solver = _shifted_solver(op, restart)
    z = complex(shift)
    info, hist, matvecs = solver.solve(z, _jacobi_inverse(op.diagonal, z), bd, x, rtol=rtol, maxiter=maxiter,
                                       use_x0=initial_solution is not None)
    op.action_calls += matvecs + 1
    true = _true_relative_residual(ops, z, x, bd, float(np.linalg.norm(b)))
    return ComponentShiftedSolution(None, 0, bool(info == 0 and true <= max(10.0 * rtol, 1.0e-12)), len(hist), true,
                                    tuple(hist), time.perf_counter() - started, solution=x.cpu().numpy(), info=info)


def _shifted_solver(op, restart: int) -> _ShiftedGMRES:
    cache = op.__dict__.setdefault("_shifted_solvers", {})
    if restart not in cache:
        cache[restart] = _ShiftedGMRES(op.context.ops, restart)
    return cache[restart]


def _retarded_green_gmres(op, add, rem, sink, freq, eta, rtol, restart, maxiter, started):
    """The reference's per-frequency loop (component_response.py:200-233) on the device."""
    ops = op.context.ops
    solver = _shifted_solver(op, restart)
    vec = DeviceVectors(ops.device)
    sink_conj = torch.conj(sink).resolve_conj().reshape(1, -1).contiguous()
    gval = torch.empty(1, dtype=torch.complex128, device=ops.device)
    out = {}
    for name, b in (("addition", add), ("removal", rem)):
        x = torch.zeros_like(b)
        bnorm = float(torch.linalg.vector_norm(b).item())
        values = np.empty(freq.size, np.complex128)
        records = []
        for i, w in enumerate(freq):
            z = complex(float(w), float(eta))
            t0 = time.perf_counter()
            info, hist, matvecs = solver.solve(z, _jacobi_inverse(op.diagonal, z), b, x, rtol=rtol, maxiter=maxiter,
                                               use_x0=i > 0)
            op.action_calls += matvecs + 1
            true = _true_relative_residual(ops, z, x, b, bnorm)
            converged = bool(info == 0 and true <= max(10.0 * rtol, 1.0e-12))
            if not converged:
                raise RuntimeError("a component EOM shifted solve failed to converge")
            vec.dots_c(sink_conj, 1, x, gval)                   # sink . x (bilinear)
            values[i] = complex(gval.item())
            records.append(ComponentShiftedSolution(None, i, converged, len(hist), true, tuple(hist),
                                                    time.perf_counter() - t0, solution=None, info=info))
        out[name] = (values, records)
    (ga, ra), (gr, rr) = out["addition"], out["removal"]
    return ComponentRetardedGreen(
        omega=freq, eta=float(eta), addition=ga, removal=gr, retarded=ga + gr,
        addition_relative_residuals=np.array([r.true_relative_residual for r in ra]),
        removal_relative_residuals=np.array([r.true_relative_residual for r in rr]),
        krylov_dimensions=(), component_action_calls=0, wall_seconds=float(time.perf_counter() - started),
        peak_rss_kib=int(resource.getrusage(resource.RUSAGE_SELF).ru_maxrss), _records_direct=(tuple(ra), tuple(rr)))


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
    _records_direct: tuple = ()

    def _records(self, which: int):
        if self._records_direct:
            return self._records_direct[which]
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
                             maxiter: int = 200, method: str = "arnoldi") -> ComponentRetardedGreen:
    """Addition and removal contributions to G^R(omega) (component_response.py:180-245).

    ``method="arnoldi"`` (default) solves every frequency from one CGS2
    Arnoldi basis per channel; ``method="gmres"`` runs the reference's own
    per-frequency loop (one preconditioned GMRES per frequency and channel,
    started from the previous frequency's solution) with the same kernels.
    """
    if method not in ("arnoldi", "gmres"):
        raise ValueError("method must be 'arnoldi' or 'gmres'")
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
    if method == "gmres":
        calls0 = op.action_calls
        res = _retarded_green_gmres(op, add.contiguous(), rem.contiguous(), sink.contiguous(), freq, eta, rtol,
                                    restart, maxiter, started)
        return dataclasses.replace(res, component_action_calls=op.action_calls - calls0)
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


# ===================================================== matrix Arnoldi response
class ArnoldiProjection:
    """One channel's projection K V_m = V_m H_m + h v_{m+1} e_m^T.

    Mirrors ``ArnoldiResolvent`` (``src/c3l/green/krylov.py:28-254``); the basis
    stays on the device (``basis`` copies it to the host on request, as the
    reference's ``[N, m+1]`` matrix).
    """

    def __init__(self, channel_basis, residual_tolerance: float, peak_rss_kib: int):
        b = channel_basis
        self._V = b.V
        self.hessenberg = b.H
        self.source_norm = np.float64(b.beta)
        self.breakdown = bool(b.breakdown)
        self.check_dimensions = tuple(int(d) for d in b.check_dimensions)
        self.check_maximum_relative_residuals = np.asarray(b.check_residuals, np.float64)
        self.residual_tolerance = np.float64(residual_tolerance)
        self.converged = bool(b.converged)
        self.construction_wall_seconds = np.float64(b.wall_seconds)
        self.action_wall_seconds = np.zeros(0, np.float64)
        self.peak_rss_kib = int(peak_rss_kib)
        self._final_residuals = b.residual

    @property
    def dimension(self) -> int:
        return int(self.hessenberg.shape[1])

    @property
    def vector_dimension(self) -> int:
        return int(self._V.shape[1])

    @property
    def terminal_coupling(self) -> complex:
        m = self.dimension
        return complex(self.hessenberg[m, m - 1])

    @property
    def basis(self) -> np.ndarray:
        return self._V[:self.dimension + 1].cpu().numpy().T

    def _dim(self, dimension):
        m = self.dimension if dimension is None else dimension
        if isinstance(m, bool) or not isinstance(m, (int, np.integer)):
            raise TypeError("dimension must be an integer")
        if not 1 <= m <= self.dimension:
            raise ValueError("dimension must lie in [1, krylov_dimension]")
        return int(m)

    def _shifts(self, shifts) -> torch.Tensor:
        z = np.asarray(shifts, dtype=np.complex128)
        if z.ndim != 1 or z.size == 0 or not np.all(np.isfinite(z)):
            raise ValueError("shifts must be a finite nonempty vector")
        return torch.from_numpy(z.copy()).to(self._V.device)

    def coefficients(self, shifts, *, dimension=None) -> np.ndarray:
        """Reduced coordinates y(z) with (z - H_m) y = |b| e_1 (device solve)."""
        m = self._dim(dimension)
        Y = hessenberg_coordinates(self.hessenberg, m, float(self.source_norm), self._shifts(shifts))
        return Y.cpu().numpy()

    def residual_norms(self, shifts, *, dimension=None) -> np.ndarray:
        m = self._dim(dimension)
        reduced = self.coefficients(shifts, dimension=m)
        return np.abs(self.hessenberg[m, m - 1] * reduced[:, -1]).astype(np.float64)

    def relative_residuals(self, shifts, *, dimension=None) -> np.ndarray:
        return self.residual_norms(shifts, dimension=dimension) / max(float(self.source_norm),
                                                                      np.finfo(np.float64).tiny)

    def solutions(self, shifts, *, dimension=None) -> np.ndarray:
        m = self._dim(dimension)
        Y = torch.from_numpy(self.coefficients(shifts, dimension=m)).to(self._V.device)
        vec = DeviceVectors(self._V.device)
        out = torch.zeros((Y.shape[0], self._V.shape[1]), dtype=torch.complex128, device=Y.device)
        for s in range(Y.shape[0]):
            vec.axpy_c(self._V, m, Y[s], 1.0, out[s])
        return out.cpu().numpy()

    def projected_rows(self, rows: torch.Tensor, m: int) -> np.ndarray:
        """P[a, k] = rows[a] . v_k (bilinear) for k < m, from the device basis."""
        vec = DeviceVectors(self._V.device)
        out = torch.empty((rows.shape[0], m), dtype=torch.complex128, device=self._V.device)
        for a in range(rows.shape[0]):
            vec.dots_c(self._V, m, torch.conj(rows[a]).resolve_conj().contiguous(), out[a])
        return np.conj(out.cpu().numpy())

    def time_coefficients(self, time, *, dimension=None) -> np.ndarray:
        """exp(-i H_m t) |b| e_1 on a time grid (``krylov.py:134-176``): SciPy's
        ``expm_multiply`` on the m x m Hessenberg matrix, one call for a uniform
        grid, one per time otherwise."""
        from scipy.sparse.linalg import expm_multiply

        t = np.asarray(time, dtype=np.float64)
        if t.ndim != 1 or t.size == 0 or not np.all(np.isfinite(t)):
            raise ValueError("time must be a finite nonempty vector")
        m = self._dim(dimension)
        H = self.hessenberg[:m, :m]
        rhs = np.zeros(m, dtype=np.complex128)
        rhs[0] = self.source_norm
        if t.size == 1:
            reduced = expm_multiply(-1j * float(t[0]) * H, rhs)[None, :]
        elif np.allclose(np.diff(t), t[1] - t[0], atol=1.0e-14, rtol=1.0e-14):
            reduced = expm_multiply(-1j * H, rhs, start=float(t[0]), stop=float(t[-1]), num=t.size, endpoint=True)
        else:
            reduced = np.asarray([expm_multiply(-1j * float(v) * H, rhs) for v in t], dtype=np.complex128)
        return np.asarray(reduced, dtype=np.complex128)

    def time_residual_norms(self, time, *, dimension=None) -> np.ndarray:
        """|h_{m+1,m} e_m^T exp(-i H_m t) |b| e_1|: the propagator's own residual."""
        m = self._dim(dimension)
        reduced = self.time_coefficients(time, dimension=m)
        return np.abs(self.hessenberg[m, m - 1] * reduced[:, -1]).astype(np.float64)

    def relative_time_residuals(self, time, *, dimension=None) -> np.ndarray:
        return self.time_residual_norms(time, dimension=dimension) / max(float(self.source_norm),
                                                                                np.finfo(np.float64).tiny)

    def transfer(self, shifts, sink, *, dimension=None) -> np.ndarray:
        """sink . x(z) at the full projection or one saved prefix (``krylov.py:210-224``)."""
        row = np.asarray(sink, dtype=np.complex128)
        if row.shape != (self.vector_dimension,) or not np.all(np.isfinite(row)):
            raise ValueError("sink must match the full vector dimension")
        m = self._dim(dimension)
        reduced = self.coefficients(shifts, dimension=m)
        rows = torch.from_numpy(row.copy()).to(self._V.device)[None, :]
        return np.asarray(reduced @ self.projected_rows(rows, m)[0], dtype=np.complex128)

    @property
    def orthogonality_defect(self) -> np.float64:
        """|V_m^H V_m - I|_F / m (``krylov.py:392-399``), formed on the device on first use."""
        if getattr(self, "_orth", None) is None:
            m = self.dimension
            vec = DeviceVectors(self._V.device)
            gram = torch.empty((m, m), dtype=torch.complex128, device=self._V.device)
            for k in range(m):
                vec.dots_c(self._V, m, self._V[k], gram[k])  # gram[k, j] = conj(v_j) . v_k
            g = gram.cpu().numpy().T
            self._orth = np.float64(np.linalg.norm(g - np.eye(m), ord="fro") / max(float(m), 1.0))
        return self._orth

    def to_dict(self) -> dict:
        return {
            "krylov_dimension": self.dimension,
            "full_vector_dimension": self.vector_dimension,
            "source_norm": float(self.source_norm),
            "terminal_coupling_absolute": float(abs(self.terminal_coupling)),
            "orthogonality_defect": float(self.orthogonality_defect),
            "action_wall_seconds": [float(v) for v in self.action_wall_seconds],
            "action_wall_seconds_total": float(np.sum(self.action_wall_seconds)),
            "construction_wall_seconds": float(self.construction_wall_seconds),
            "peak_rss_kib": self.peak_rss_kib,
            "breakdown": self.breakdown,
            "check_dimensions": list(self.check_dimensions),
            "check_maximum_relative_residuals": [float(v) for v in self.check_maximum_relative_residuals],
            "maximum_relative_residual": float(self.check_maximum_relative_residuals[-1]),
            "residual_tolerance": float(self.residual_tolerance),
            "converged": self.converged,
            "method": "two_pass_one_sided_Arnoldi_shift_invariant_resolvent",
        }


@dataclass(frozen=True)
class ComponentRetardedMatrixArnoldiGreen:
    omega: np.ndarray
    eta: float
    sites: tuple
    addition: np.ndarray
    removal: np.ndarray
    retarded: np.ndarray
    addition_projections: tuple
    removal_projections: tuple
    addition_relative_residuals: np.ndarray
    removal_relative_residuals: np.ndarray
    component_action_calls: int
    component_action_wall_seconds: float
    wall_seconds: float
    peak_rss_kib: int


def _validated_source_columns(operator, sources):
    """component_response.py:496-516"""
    columns = tuple(sources)
    if not columns:
        raise ValueError("at least one impurity source is required")
    if len({item.site for item in columns}) != len(columns):
        raise ValueError("impurity source sites must be unique")
    if any(item.charge != columns[0].charge for item in columns):
        raise ValueError("all impurity sources must use one response charge")
    retained = np.asarray(columns[0].addition).size
    for item in columns:
        if (np.asarray(item.addition).shape != (retained,) or np.asarray(item.removal).shape != (retained,)
                or np.asarray(item.sink).shape != (retained,)):
            raise ValueError("impurity sources and sinks must share one retained basis")
    if operator.dimension < retained:
        raise ValueError("response operator is smaller than the retained sources")
    return columns, retained


def _validated_krylov_controls(operator, maximum, minimum, interval, tolerance):
    """component_response.py:519-547"""
    for v in (maximum, minimum, interval):
        if isinstance(v, bool) or not isinstance(v, (int, np.integer)):
            raise TypeError("Krylov dimensions and check_interval must be integers")
    if maximum <= 0 or minimum <= 0 or interval <= 0 or not np.isfinite(tolerance) or tolerance <= 0.0:
        raise ValueError("Krylov controls and residual tolerance must be positive")
    maximum_dimension = int(min(maximum, operator.dimension, 4096))
    minimum_dimension = int(min(minimum, maximum_dimension))
    return maximum_dimension, minimum_dimension


def component_retarded_matrix_green_arnoldi(operator, sources, omega, eta: float, *,
                                            maximum_krylov_dimension: int = 320,
                                            residual_tolerance: float = 1.0e-10,
                                            minimum_krylov_dimension: int = 16,
                                            check_interval: int = 8) -> ComponentRetardedMatrixArnoldiGreen:
    """G^R_ab(omega) for every sink a and source b from one Arnoldi basis per source and channel.

    Same inputs, controls, errors and result fields as the reference
    (``src/c3l/cc/component_response.py:356-423``).  All 2 x len(sources)
    channels run concurrently (one stream and sigma workspace each); for
    channel b, ``values[:, a, b] = Y(z) (sink_a . V_m)^T`` with the reduced
    coordinates Y solved on the device for every shift.
    """
    started = time.perf_counter()
    if not hasattr(operator, "action_calls"):
        raise TypeError("operator must be an instrumented ComponentSigmaOperator")
    columns, retained = _validated_source_columns(operator, sources)
    frequency = np.asarray(omega, dtype=np.float64)
    broadening = float(eta)
    if (frequency.ndim != 1 or frequency.size == 0 or not np.all(np.isfinite(frequency))
            or not np.isfinite(broadening) or broadening <= 0.0):
        raise ValueError("omega and positive eta must be finite")
    max_dim, min_dim = _validated_krylov_controls(operator, maximum_krylov_dimension, minimum_krylov_dimension,
                                                  check_interval, residual_tolerance)
    r = _matrix_arnoldi_response(operator, columns, (frequency + 1j * broadening).astype(np.complex128),
                                 max_dim, min_dim, float(residual_tolerance), int(check_interval))
    return ComponentRetardedMatrixArnoldiGreen(
        omega=frequency, eta=broadening, sites=r["sites"], addition=r["values"][0], removal=r["values"][1],
        retarded=r["values"][0] + r["values"][1], addition_projections=r["projections"][0],
        removal_projections=r["projections"][1], addition_relative_residuals=r["residuals"][0],
        removal_relative_residuals=r["residuals"][1], component_action_calls=r["calls"],
        component_action_wall_seconds=r["action_seconds"], wall_seconds=float(time.perf_counter() - started),
        peak_rss_kib=r["rss"])


def _padded_source(item, which: int, N: int, dev) -> torch.Tensor:
    """Addition (0), removal (1) or sink (2) of a source column on the device, zero-padded to N."""
    if item.device:
        v = item.device[which]
    else:
        v = torch.from_numpy(np.asarray((item.addition, item.removal, item.sink)[which], np.complex128).copy()).to(dev)
    if v.numel() < N:
        v = torch.cat([v, torch.zeros(N - v.numel(), dtype=torch.complex128, device=dev)])
    return v.contiguous()


def _matrix_arnoldi_response(operator, columns, shifts: np.ndarray, max_dim: int, min_dim: int, tolerance: float,
                             interval: int) -> dict:
    """One Arnoldi basis per source and channel, all channels concurrent, every sink
    row contracted from each basis (``component_response.py:550-625``): for channel
    b, ``values[:, a, b] = Y(z) (sink_a . V_m)^T`` with the reduced coordinates Y
    solved on the device for every shift."""
    ops = operator.context.ops
    dev = ops.device
    N = operator.dimension
    vectors = []
    for item in columns:
        vectors += [_padded_source(item, 0, N, dev), _padded_source(item, 1, N, dev)]
    sinks = [_padded_source(item, 2, N, dev) for item in columns]
    z = torch.from_numpy(np.ascontiguousarray(shifts, dtype=np.complex128)).to(dev)
    action_seconds0 = operator.action_wall_seconds
    t_action = time.perf_counter()
    bases = arnoldi_channels(ops, vectors, z, maximum_dimension=max_dim, residual_tolerance=tolerance,
                             minimum_dimension=min_dim, check_interval=interval)
    calls = sum(b.m for b in bases)
    operator.action_calls += calls
    operator.action_wall_seconds += time.perf_counter() - t_action
    if not all(b.converged for b in bases):
        raise RuntimeError("a component EOM matrix Arnoldi projection failed")
    S = len(columns)
    ns = shifts.size
    values = [np.empty((ns, S, S), np.complex128), np.empty((ns, S, S), np.complex128)]
    residuals = [np.empty((S, ns), np.float64), np.empty((S, ns), np.float64)]
    vec = DeviceVectors(dev)
    sink_conj = [torch.conj(s).resolve_conj().contiguous() for s in sinks]
    for idx, basis in enumerate(bases):
        b, kind = divmod(idx, 2)
        m = basis.m
        Y = reduced_coordinates(basis, z)                          # [ns, m]
        for a in range(S):
            # p_k = sink_a . v_k (bilinear), then values[s, a, b] = sum_k Y[s, k] p_k
            pc = torch.empty(m, dtype=torch.complex128, device=dev)
            vec.dots_c(basis.V, m, sink_conj[a], pc)               # conj(p)
            g = torch.empty(ns, dtype=torch.complex128, device=dev)
            vec.dots_c(Y, ns, pc, g)                               # conj(sum_k Y p)
            values[kind][:, a, b] = np.conj(g.cpu().numpy())
        residuals[kind][b] = basis.residual.cpu().numpy()
    rss = int(resource.getrusage(resource.RUSAGE_SELF).ru_maxrss)
    proj = [ArnoldiProjection(bb, tolerance, rss) for bb in bases]
    return {"sites": tuple(int(item.site) for item in columns), "values": values, "residuals": residuals,
            "projections": (tuple(proj[0::2]), tuple(proj[1::2])), "calls": int(calls),
            "action_seconds": float(operator.action_wall_seconds - action_seconds0), "rss": rss}


@dataclass(frozen=True)
class ComponentShiftedMatrixArnoldiGreen:
    """``retarded[k, a, b]`` = G^R_ab(z_k), sink a, source b (``component_response.py:427-446``)."""
    shifts: np.ndarray
    sites: tuple
    addition: np.ndarray
    removal: np.ndarray
    retarded: np.ndarray
    addition_projections: tuple
    removal_projections: tuple
    addition_relative_residuals: np.ndarray
    removal_relative_residuals: np.ndarray
    action_calls: int
    wall_seconds: float
    peak_rss_kib: int


def component_retarded_matrix_green_shifts(operator, sources, shifts, *, maximum_krylov_dimension: int = 320,
                                           residual_tolerance: float = 1.0e-10, minimum_krylov_dimension: int = 16,
                                           check_interval: int = 8) -> ComponentShiftedMatrixArnoldiGreen:
    """G^R(z) at complex shifts with Im z > 0 (``component_response.py:449-493``):
    the matrix Arnoldi response without the omega + i eta restriction, so
    imaginary-axis points share one Krylov space per source with real-axis
    points.  Same inputs, controls, errors and result fields as the reference."""
    started = time.perf_counter()
    if not hasattr(operator, "action_calls"):
        raise TypeError("operator must be an instrumented ComponentSigmaOperator")
    columns, _ = _validated_source_columns(operator, sources)
    z = np.asarray(shifts, dtype=np.complex128)
    if z.ndim != 1 or z.size == 0 or not np.all(np.isfinite(z)) or np.any(z.imag <= 0.0):
        raise ValueError("shifts must be finite with positive imaginary parts")
    max_dim, min_dim = _validated_krylov_controls(operator, maximum_krylov_dimension, minimum_krylov_dimension,
                                                  check_interval, residual_tolerance)
    r = _matrix_arnoldi_response(operator, columns, z, max_dim, min_dim, float(residual_tolerance),
                                 int(check_interval))
    return ComponentShiftedMatrixArnoldiGreen(
        shifts=np.asarray(z, dtype=np.complex128), sites=r["sites"], addition=r["values"][0],
        removal=r["values"][1], retarded=r["values"][0] + r["values"][1], addition_projections=r["projections"][0],
        removal_projections=r["projections"][1], addition_relative_residuals=r["residuals"][0],
        removal_relative_residuals=r["residuals"][1], action_calls=r["calls"],
        wall_seconds=float(time.perf_counter() - started), peak_rss_kib=r["rss"])


# ============================================================ time domain
def _arnoldi_projections(operator, vectors, shifts: np.ndarray, max_dim: int, tolerance: float):
    """``arnoldi_resolvent`` with the time drivers' controls (minimum dimension
    min(16, N), check interval min(8, N)) for several source vectors at once;
    one action call per basis vector, as the reference counts them."""
    ops = operator.context.ops
    N = operator.dimension
    z = torch.from_numpy(np.ascontiguousarray(shifts, dtype=np.complex128)).to(ops.device)
    t0 = time.perf_counter()
    bases = arnoldi_channels(ops, vectors, z, maximum_dimension=max_dim, residual_tolerance=tolerance,
                             minimum_dimension=min(16, N), check_interval=min(8, N))
    operator.action_calls += sum(b.m for b in bases)
    operator.action_wall_seconds += time.perf_counter() - t0
    rss = int(resource.getrusage(resource.RUSAGE_SELF).ru_maxrss)
    return [ArnoldiProjection(b, tolerance, rss) for b in bases]


def component_retarded_time(operator, sources, time, *, maximum_krylov_dimension: int = 160,
                            residual_tolerance: float = 1.0e-11) -> np.ndarray:
    """-i sink . exp(-i K t) (addition + removal) for t >= 0 (``component_response.py:628-663``).

    One Arnoldi basis of the combined source (stopping test at the probe shift
    z = i, as in the reference) is built on the device; the propagator acts on
    the m x m Hessenberg matrix (SciPy's ``expm`` per time, as the reference).
    """
    from scipy.linalg import expm

    t = np.asarray(time, dtype=np.float64)
    N = operator.dimension
    dev = operator.context.ops.device
    source = _padded_source(sources, 0, N, dev) + _padded_source(sources, 1, N, dev)
    sink = _padded_source(sources, 2, N, dev)
    proj = _arnoldi_projections(operator, [source.contiguous()], np.asarray([1j], np.complex128),
                                int(min(maximum_krylov_dimension, N)), float(residual_tolerance))[0]
    m = proj.dimension
    H = proj.hessenberg[:m, :m]
    reduced_source = np.zeros(m, dtype=np.complex128)
    reduced_source[0] = proj.source_norm
    projected_sink = proj.projected_rows(sink[None, :], m)[0]
    out = np.empty(t.size, dtype=np.complex128)
    for i, value in enumerate(t):
        out[i] = -1j * (projected_sink @ (expm(-1j * float(value) * H) @ reduced_source))
    return out


@dataclass(frozen=True)
class ComponentRetardedMatrixTime:
    """Direct-time impurity Green matrix from one basis per source column (``component_response.py:666-682``)."""
    time: np.ndarray
    sites: tuple
    addition: np.ndarray
    removal: np.ndarray
    retarded: np.ndarray
    channel_sum_defect: float
    combined_projections: tuple
    addition_projections: tuple
    removal_projections: tuple
    combined_relative_time_residuals: np.ndarray
    addition_relative_time_residuals: np.ndarray
    removal_relative_time_residuals: np.ndarray
    wall_seconds: float
    peak_rss_kib: int


def _matrix_time_from_projections(projections, sinks: torch.Tensor, t: np.ndarray) -> np.ndarray:
    """out[:, a, b] = -i exp(-i H t) |b| e_1 . (sink_a . V_m) (``component_response.py:685-699``)."""
    out = np.empty((t.size, sinks.shape[0], len(projections)), dtype=np.complex128)
    for b, proj in enumerate(projections):
        m = proj.dimension
        projected = proj.projected_rows(sinks, m)              # [S, m]
        out[:, :, b] = -1j * (proj.time_coefficients(t) @ projected.T)
    return out


def component_retarded_matrix_time(operator, sources, time, validation_shifts, *,
                                   maximum_krylov_dimension: int = 160, residual_tolerance: float = 1.0e-11,
                                   include_channels: bool = True) -> ComponentRetardedMatrixTime:
    """All sink rows from one combined-source basis per source orbital, plus the
    separate addition/removal bases when ``include_channels`` (the channel-sum
    diagnostic).  Same inputs, errors and result fields as the reference
    (``component_response.py:702-815``); all bases run as concurrent device
    channels."""
    started = perf_counter()
    columns, _ = _validated_source_columns(operator, sources)
    t = np.asarray(time, dtype=np.float64)
    z = np.asarray(validation_shifts, dtype=np.complex128)
    if (t.ndim != 1 or t.size == 0 or np.any(t < 0.0) or not np.all(np.isfinite(t)) or z.ndim != 1 or z.size == 0
            or not np.all(np.isfinite(z))):
        raise ValueError("time and validation shifts must be finite nonempty vectors")
    N = operator.dimension
    dev = operator.context.ops.device
    sinks = torch.stack([_padded_source(item, 2, N, dev) for item in columns])
    vectors = [(_padded_source(item, 0, N, dev) + _padded_source(item, 1, N, dev)).contiguous() for item in columns]
    if include_channels:
        vectors += [_padded_source(item, 0, N, dev) for item in columns]
        vectors += [_padded_source(item, 1, N, dev) for item in columns]
    proj = _arnoldi_projections(operator, vectors, z, int(min(maximum_krylov_dimension, N)),
                                float(residual_tolerance))
    S = len(columns)
    combined = tuple(proj[:S])
    retarded = _matrix_time_from_projections(combined, sinks, t)
    combined_res = np.asarray([p.relative_time_residuals(t) for p in combined], dtype=np.float64)
    if include_channels:
        add_p, rem_p = tuple(proj[S:2 * S]), tuple(proj[2 * S:])
        addition = _matrix_time_from_projections(add_p, sinks, t)
        removal = _matrix_time_from_projections(rem_p, sinks, t)
        add_res = np.asarray([p.relative_time_residuals(t) for p in add_p], dtype=np.float64)
        rem_res = np.asarray([p.relative_time_residuals(t) for p in rem_p], dtype=np.float64)
        defect = float(np.max(abs(retarded - addition - removal)))
    else:
        add_p = rem_p = ()
        add_res = np.empty((0, t.size), dtype=np.float64)
        rem_res = np.empty((0, t.size), dtype=np.float64)
        addition = np.full_like(retarded, np.nan + 1j * np.nan)
        removal = np.full_like(retarded, np.nan + 1j * np.nan)
        defect = float("nan")
    return ComponentRetardedMatrixTime(
        time=t, sites=tuple(int(item.site) for item in columns), addition=addition, removal=removal,
        retarded=retarded, channel_sum_defect=defect, combined_projections=combined, addition_projections=add_p,
        removal_projections=rem_p, combined_relative_time_residuals=combined_res,
        addition_relative_time_residuals=add_res, removal_relative_time_residuals=rem_res,
        wall_seconds=float(perf_counter() - started),
        peak_rss_kib=int(resource.getrusage(resource.RUSAGE_SELF).ru_maxrss))


# ============================================= matrix response, GMRES form
@dataclass(frozen=True)
class ComponentRetardedMatrixGreen:
    """Frequency-domain Green matrix from one response solve per source column
    and frequency (``component_response.py:145-158``)."""
    omega: np.ndarray
    eta: float
    sites: tuple
    addition: np.ndarray
    removal: np.ndarray
    retarded: np.ndarray
    addition_solutions: tuple
    removal_solutions: tuple
    wall_seconds: float
    peak_rss_kib: int


def component_retarded_matrix_green(operator, sources, omega, eta: float, *, rtol: float = 1.0e-10,
                                    restart: int = 40, maxiter: int = 200) -> ComponentRetardedMatrixGreen:
    """All sink rows with one addition/removal solve per source column and frequency
    (``component_response.py:248-353``): preconditioned restarted GMRES on the
    device (``c3l_gmres_shifted``), each frequency started from the previous
    frequency's solution, every sink contracted with the same solutions.  Axes
    ``(omega, sink_site, source_site)``; a solve that misses the convergence
    rule of ``solve_component_shifted`` raises."""
    columns, _ = _validated_source_columns(operator, sources)
    frequency = np.asarray(omega, dtype=np.float64)
    broadening = float(eta)
    if (frequency.ndim != 1 or frequency.size == 0 or not np.all(np.isfinite(frequency))
            or not np.isfinite(broadening) or broadening <= 0.0):
        raise ValueError("omega and positive eta must be finite")
    op = operator if isinstance(operator, ComponentSigmaOperator) else ComponentSigmaOperator(operator)
    ops = op.context.ops
    dev = ops.device
    N = op.dimension
    S = len(columns)
    started = time.perf_counter()
    sinks_conj = torch.stack([torch.conj(_padded_source(item, 2, N, dev)).resolve_conj() for item in columns])
    shape = (frequency.size, S, S)
    values = [np.empty(shape, np.complex128), np.empty(shape, np.complex128)]
    records = [[], []]
    solver = _shifted_solver(op, restart)
    vec = DeviceVectors(dev)
    row = torch.empty(S, dtype=torch.complex128, device=dev)
    for b, item in enumerate(columns):
        for kind in (0, 1):
            rhs = _padded_source(item, kind, N, dev)
            bnorm = float(torch.linalg.vector_norm(rhs).item())
            x = torch.zeros_like(rhs)
            per = []
            for i, w in enumerate(frequency):
                z = complex(float(w), broadening)
                t0 = time.perf_counter()
                info, hist, matvecs = solver.solve(z, _jacobi_inverse(op.diagonal, z), rhs, x, rtol=rtol,
                                                   maxiter=maxiter, use_x0=i > 0)
                op.action_calls += matvecs + 1
                true = _true_relative_residual(ops, z, x, rhs, bnorm)
                converged = bool(info == 0 and true <= max(10.0 * rtol, 1.0e-12))
                if not converged:
                    raise RuntimeError("a component EOM matrix shifted solve failed")
                vec.dots_c(sinks_conj, S, x, row)                 # sink_a . x (bilinear)
                values[kind][i, :, b] = row.cpu().numpy()
                per.append(ComponentShiftedSolution(None, i, converged, len(hist), true, tuple(hist),
                                                    time.perf_counter() - t0, solution=x.cpu().numpy(), info=info))
            records[kind].append(tuple(per))
    return ComponentRetardedMatrixGreen(
        omega=frequency, eta=broadening, sites=tuple(int(item.site) for item in columns), addition=values[0],
        removal=values[1], retarded=values[0] + values[1], addition_solutions=tuple(records[0]),
        removal_solutions=tuple(records[1]), wall_seconds=float(time.perf_counter() - started),
        peak_rss_kib=int(resource.getrusage(resource.RUSAGE_SELF).ru_maxrss))
