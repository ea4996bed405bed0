"""Static CCSD on the GPU: problem, residual/JVP actions and Newton--Krylov.

Drop-in counterparts of the reference's
``ComponentStaticProblem`` (``src/c3l/cc/component_tensor.py:1254-1298``),
``component_static_residual`` / ``component_static_jvp`` (``:1822-1930``),
``NewtonKrylovPolicy`` (``src/c3l/cc/newton_krylov.py:35-123``) and
``solve_component_ccsd`` (``src/c3l/cc/component_solver.py:103-295``).
"""

from __future__ import annotations

import dataclasses
import resource
import time
from dataclasses import dataclass, field
from pathlib import Path
from typing import Callable

import numpy as np
import torch

from . import runtime as rt
from .krylov import DeviceGMRES, DeviceVectors
from .spec import ProblemSpec


# ------------------------------------------------------------------ policy
@dataclass(frozen=True, slots=True)
class NewtonKrylovPolicy:
    """Numerical controls of the static solve (same fields and rules as the reference)."""

    tolerance: float = 1.0e-10
    maximum_newton_iterations: int = 20
    gmres_restart: int = 40
    gmres_maximum_restart_cycles: int = 12
    minimum_gmres_relative_tolerance: float = 1.0e-8
    maximum_gmres_relative_tolerance: float = 1.0e-3
    maximum_line_search_steps: int = 14
    armijo: float = 1.0e-4
    forcing_strategy: str = "legacy"
    initial_gmres_relative_tolerance: float = 1.0e-2
    eisenstat_walker_gamma: float = 0.9
    eisenstat_walker_exponent: float = 1.5
    gmres_absolute_tolerance_factor: float = 0.1

    def __post_init__(self) -> None:
        pos = (self.tolerance, self.minimum_gmres_relative_tolerance, self.maximum_gmres_relative_tolerance,
               self.armijo, self.initial_gmres_relative_tolerance, self.eisenstat_walker_gamma,
               self.eisenstat_walker_exponent, self.gmres_absolute_tolerance_factor)
        if not all(np.isfinite(v) and v > 0.0 for v in pos):
            raise ValueError("Newton--Krylov tolerances must be finite and positive")
        if self.minimum_gmres_relative_tolerance > self.maximum_gmres_relative_tolerance:
            raise ValueError("minimum GMRES tolerance exceeds the maximum")
        if self.maximum_gmres_relative_tolerance >= 1.0 or self.armijo >= 1.0:
            raise ValueError("relative and Armijo tolerances must be smaller than one")
        if self.forcing_strategy not in ("legacy", "eisenstat_walker"):
            raise ValueError("unknown inexact-Newton forcing strategy")
        if not 0.0 < self.eisenstat_walker_gamma < 1.0:
            raise ValueError("Eisenstat--Walker gamma must lie in (0,1)")
        if not 1.0 < self.eisenstat_walker_exponent <= 2.0:
            raise ValueError("Eisenstat--Walker exponent must lie in (1,2]")
        if not 0.0 < self.gmres_absolute_tolerance_factor <= 1.0:
            raise ValueError("GMRES absolute-tolerance factor must lie in (0,1]")
        if self.forcing_strategy == "eisenstat_walker" and not (
                self.minimum_gmres_relative_tolerance <= self.initial_gmres_relative_tolerance
                <= self.maximum_gmres_relative_tolerance):
            raise ValueError("initial GMRES tolerance lies outside the forcing bounds")
        for v in (self.maximum_newton_iterations, self.gmres_restart, self.gmres_maximum_restart_cycles,
                  self.maximum_line_search_steps):
            if isinstance(v, bool) or not isinstance(v, int) or v <= 0:
                raise ValueError("Newton--Krylov iteration limits must be positive integers")

    def to_dict(self) -> dict:
        out = {k: getattr(self, k) for k in (
            "tolerance", "maximum_newton_iterations", "gmres_restart", "gmres_maximum_restart_cycles",
            "minimum_gmres_relative_tolerance", "maximum_gmres_relative_tolerance", "maximum_line_search_steps",
            "armijo")}
        if self.forcing_strategy == "eisenstat_walker":
            out.update({k: getattr(self, k) for k in (
                "forcing_strategy", "initial_gmres_relative_tolerance", "eisenstat_walker_gamma",
                "eisenstat_walker_exponent", "gmres_absolute_tolerance_factor")})
        return out


def forcing_tolerance(norm: float, policy: NewtonKrylovPolicy, *, previous_norm=None, previous_tolerance=None) -> float:
    """Relative linear defect requested per Newton step (newton_krylov.py:209-237)."""
    if policy.forcing_strategy == "legacy":
        value = 0.1 * max(norm, policy.tolerance)
    elif previous_norm is None:
        value = policy.initial_gmres_relative_tolerance
    else:
        ratio = norm / max(previous_norm, np.finfo(float).tiny)
        value = policy.eisenstat_walker_gamma * ratio ** policy.eisenstat_walker_exponent
        if previous_tolerance is not None:
            value = max(value, policy.eisenstat_walker_gamma * previous_tolerance ** policy.eisenstat_walker_exponent)
    return float(min(policy.maximum_gmres_relative_tolerance, max(policy.minimum_gmres_relative_tolerance, value)))


@dataclass(frozen=True, slots=True)
class NewtonKrylovStep:
    iteration: int
    residual_norm: float
    gmres_relative_tolerance: float
    gmres_info: int
    gmres_iterations: int
    gmres_preconditioned_residual_history: tuple
    true_linear_relative_residual: float
    step_norm: float
    damping: float
    accepted_residual_norm: float


@dataclass(frozen=True, slots=True)
class RapidityPreconditionerDiagnostics:
    minimum_magnitude: float
    maximum_magnitude: float
    magnitude_condition: float
    regularization_threshold: float
    regularized_amplitudes: int


@dataclass(frozen=True, slots=True)
class ComponentStaticAction:
    retained: np.ndarray
    reference: complex
    wall_seconds: float
    materialization: object = None


@dataclass(frozen=True, slots=True)
class ComponentCCSolution:
    problem: object
    variables: np.ndarray
    amplitudes: np.ndarray
    residual: ComponentStaticAction
    residual_norm: float
    packed_residual_norm: float
    reference_residual: float
    rank6: object
    converged: bool
    iterations: int
    residual_evaluations: int
    jvp_evaluations: int
    history: tuple
    preconditioner: RapidityPreconditionerDiagnostics
    wall_seconds: float
    peak_rss_kib: int
    gpu_launches: int = 0
    warm_start: str = "none"
    # the amplitudes as the device vector they were unpacked into (an EOM
    # context built from it needs no host round trip)
    device_amplitudes: object = field(default=None, repr=False, compare=False)
    # the homotopy scale of the model these amplitudes solve (1: the problem as compiled)
    interaction_scale: float = 1.0


# ----------------------------------------------------------------- problem
def _is_reference_object(obj) -> bool:
    return type(obj).__module__.startswith("c3l.")


class ComponentStaticProblem:
    """GPU-resident factorized CCSD problem.

    ``compile`` accepts a ``ProblemSpec`` (or a path to one), the reference's
    ``FactorizedCCProblem`` or the reference's ``ComponentStaticProblem``.
    The device program is compiled lazily on first use.
    """

    def __init__(self, spec: ProblemSpec, *, device=None, oracle=None):
        self.spec = spec
        self.oracle = oracle
        self._device = device
        self._plan = None
        self._ops = None

    @classmethod
    def compile(cls, problem, *, fuse_products: bool = False, device=None) -> "ComponentStaticProblem":
        if isinstance(problem, ComponentStaticProblem):
            return problem
        if isinstance(problem, ProblemSpec):
            return cls(problem, device=device)
        if isinstance(problem, (str, Path)):
            return cls(ProblemSpec.load(problem), device=device)
        if _is_reference_object(problem):
            cc = problem.oracle if hasattr(problem, "coordinates") else problem
            if getattr(cc, "level", "CCSD") != "CCSD":
                raise ValueError("the component backend currently implements CCSD only")
            return cls(ProblemSpec.from_factorized(cc), device=device, oracle=cc)
        raise TypeError("unsupported problem type")

    @property
    def plan(self):
        if self._plan is None:
            from .plans import StaticPlan
            self._plan = StaticPlan(self.spec)
        return self._plan

    @property
    def ops(self):
        if self._ops is None:
            from .device_ops import DeviceStatic
            self._ops = DeviceStatic(self.plan, self._device)
        return self._ops

    @property
    def device(self) -> torch.device:
        return self.ops.device

    def gmres_solver(self, restart: int):
        """Device GMRES buffers sized for ``restart`` (cached per restart length)."""
        cache = self.__dict__.setdefault("_gmres", {})
        if restart not in cache:
            cache[restart] = DeviceGMRES(self.ops, restart)
        return cache[restart]

    @property
    def n(self) -> int:
        return self.spec.n

    @property
    def num_amplitudes(self) -> int:
        return self.plan.num_amplitudes

    @property
    def num_variables(self) -> int:
        return self.plan.num_variables

    # boundary conversions (reference vector layouts)
    def pack(self, amplitudes) -> np.ndarray:
        """Real tilde coordinates of a tilde-invariant amplitude vector (symmetry.py:87-106)."""
        t = np.asarray(amplitudes, dtype=np.complex128)
        if t.shape != (self.num_amplitudes,) or not np.all(np.isfinite(t)):
            raise ValueError("initial amplitudes do not match the component CCSD problem")
        tl = self.plan.tilde
        x = np.empty(self.num_variables)
        v = t[tl.rep_pos] * tl.rep_scale
        x[tl.rep_col] = v.real
        pr = tl.rep_pair == 1
        x[tl.rep_col[pr] + 1] = t[tl.rep_pos[pr]].imag
        return x


def _as_problem(problem) -> ComponentStaticProblem:
    return ComponentStaticProblem.compile(problem)


def _to_device_complex(values, n: int, device, what: str) -> torch.Tensor:
    arr = np.asarray(values, dtype=np.complex128)
    if arr.shape != (n,) or not np.all(np.isfinite(arr)):
        raise ValueError(f"{what} has the wrong shape or is nonfinite")
    return torch.from_numpy(arr.copy()).to(device)


def component_static_residual(problem, amplitudes) -> ComponentStaticAction:
    """Retained residual -i pack(Lambda T + V) for arbitrary complex amplitudes."""
    p = _as_problem(problem)
    ops = p.ops
    started = time.perf_counter()
    t = _to_device_complex(amplitudes, p.num_amplitudes, ops.device, "component vector")
    out = torch.empty(p.num_amplitudes, dtype=torch.complex128, device=ops.device)
    ref = ops.residual_complex(t, out)
    host = out.cpu().numpy()
    return ComponentStaticAction(host, ref, time.perf_counter() - started)


def component_static_jvp(problem, amplitudes, direction) -> ComponentStaticAction:
    """Exact forward tangent of the residual at ``amplitudes`` along ``direction``."""
    p = _as_problem(problem)
    ops = p.ops
    started = time.perf_counter()
    t = _to_device_complex(amplitudes, p.num_amplitudes, ops.device, "component vector")
    v = _to_device_complex(direction, p.num_amplitudes, ops.device, "component direction")
    out = torch.empty(p.num_amplitudes, dtype=torch.complex128, device=ops.device)
    ref = ops.jvp_complex(t, v, out)
    return ComponentStaticAction(out.cpu().numpy(), ref, time.perf_counter() - started)


# ------------------------------------------------------------------ solver
def _acceptable_inexact_newton_step(r_norm: float, merit_slope: float, defect_norm: float, *, relative_tolerance: float,
                                    absolute_tolerance: float) -> bool:
    """True-defect and merit-descent test (component_solver.py:77-100)."""
    target = max(relative_tolerance * r_norm, absolute_tolerance)
    margin = 1.0 + np.sqrt(np.finfo(float).eps)
    return bool(np.isfinite(defect_norm) and defect_norm <= margin * target and np.isfinite(merit_slope)
                and merit_slope < 0.0)


# Mixed precision: the inner solves (FP32 JVP, FP32 Krylov basis) are asked
# for no more than this relative defect; the FP64 residual of the outer
# Newton loop supplies the remaining digits.  The FP32 basis keeps its
# Arnoldi relation to about eps_fp32 |w| / h, which slows restarted GMRES
# near 1e-6 (siam10 last step: 400 instead of 299 iterations); at 1e-5 the
# last step still leaves the Newton residual near 2e-13, far below the
# 1e-10 convergence test.
MIXED_GMRES_FLOOR = 1.0e-5
# Mixed precision, last steps: the inner solve needs to shrink the residual only
# to the outer tolerance, so a step whose residual is already near it may stop
# at MIXED_TARGET_SAFETY * tolerance / |r| (capped by the policy's largest
# relative tolerance).  The FP64 residual still decides convergence; a step
# that falls short is followed by another Newton step.
MIXED_TARGET_SAFETY = 0.05
# GMRES bases larger than this are released when a solve returns (a 960-vector
# basis of a 65-site problem holds 102 GB); smaller ones stay for the next solve.
KEEP_GMRES_BYTES = 8 << 30


def solve_component_ccsd(problem, initial_amplitudes=None, *, policy: NewtonKrylovPolicy | None = None,
                         rank6_tile_size: int = 4096, compute_rank6: bool = False,
                         accepted_step_callback: Callable | None = None, warm_start=None,
                         precision: str = "fp64", interaction_scale: float = 1.0) -> ComponentCCSolution:
    """Solve the tilde-real CCSD equations with device residuals and JVPs.

    Control flow, forcing terms, Armijo backtracking and the final
    independent residual follow ``src/c3l/cc/component_solver.py:103-295``.
    ``warm_start`` optionally supplies a learned initial guess (see
    ``c3lindblad_gb300.warmstart``); it is ignored when
    ``initial_amplitudes`` is given, and convergence of the plain residual
    decides the answer either way.

    ``precision="mixed"`` applies the JVP inside GMRES with FP32 contractions
    and keeps the GMRES basis in FP32 (the GMRES tolerance is floored at
    ``MIXED_GMRES_FLOOR`` and may rise to ``MIXED_TARGET_SAFETY`` times the
    outer tolerance over |r| near convergence) while every residual, the
    line search and the true linear defect stay FP64 -- iterative refinement,
    so the converged amplitudes meet the same FP64 residual tolerance.

    ``interaction_scale`` s solves the reference's homotopy model
    ``L0(K_ref) + s [L - L0(K_ref)]`` at the problem's own HF reference
    (``src/c3l/models.py:516-549``): the same products with every coefficient
    times s, so the compiled program is reused with its product part scaled.
    """
    if precision not in ("fp64", "mixed"):
        raise ValueError("precision must be 'fp64' or 'mixed'")
    mixed = precision == "mixed"
    if compute_rank6:
        raise NotImplementedError("the rank-six truncation diagnostic is not part of the GPU path")
    controls = NewtonKrylovPolicy() if policy is None else policy
    p = _as_problem(problem)
    ops = p.ops
    ops.set_interaction_scale(interaction_scale)
    try:
        sol = _solve(p, ops, controls, initial_amplitudes, accepted_step_callback, warm_start, precision)
        return dataclasses.replace(sol, interaction_scale=float(interaction_scale))
    finally:
        ops.set_interaction_scale(1.0)
        for key, solver in list(p.__dict__.get("_gmres", {}).items()):
            if solver.nbytes > KEEP_GMRES_BYTES:
                solver.release_graphs()
                del p.__dict__["_gmres"][key]


def _solve(p, ops, controls, initial_amplitudes, accepted_step_callback, warm_start, precision):
    mixed = precision == "mixed"
    dev = ops.device
    vec = DeviceVectors(dev)
    started = time.perf_counter()
    launches0 = rt.LaunchCounter.count
    D = p.num_variables
    warm_label = "none"
    if initial_amplitudes is not None:
        x = torch.from_numpy(p.pack(initial_amplitudes)).to(dev)
    elif warm_start is not None:
        # the learned guess is kept only if its FP64 residual beats the zero guess
        x = warm_start.initial_variables(p)
        rw = torch.empty(D, dtype=torch.float64, device=dev)
        ops.residual(x, rw)
        zero = torch.zeros(D, dtype=torch.float64, device=dev)
        r0 = torch.empty(D, dtype=torch.float64, device=dev)
        ops.residual(zero, r0)
        if vec.norm_r(rw) < vec.norm_r(r0):
            warm_label = getattr(warm_start, "label", "learned")
        else:
            x = zero
            warm_label = "rejected"
    else:
        x = torch.zeros(D, dtype=torch.float64, device=dev)
    pre = RapidityPreconditionerDiagnostics(**ops.preconditioner_diagnostics)
    r = torch.empty(D, dtype=torch.float64, device=dev)
    trial = torch.empty(D, dtype=torch.float64, device=dev)
    jstep = torch.empty(D, dtype=torch.float64, device=dev)
    scal = torch.empty(2, dtype=torch.float64, device=dev)
    residual_evaluations = 0
    jvp_evaluations = 0
    history: list = []
    converged = False
    prev_norm = None
    prev_tol = None
    jvp_count = [0]
    solver = p.gmres_solver(controls.gmres_restart)
    step = torch.empty(D, dtype=torch.float64, device=dev)
    negr = torch.empty(D, dtype=torch.float64, device=dev)

    def matvec(v, out):
        jvp_count[0] += 1
        ops.jvp(v, out)

    from .device_ops import pair_kernel_setting

    for iteration in range(controls.maximum_newton_iterations + 1):
        ops.linearize(x, r)
        residual_evaluations += 1
        if mixed:
            ops.to_single()
            if ops.pair_tuning is None and pair_kernel_setting() == "auto":
                ops.tune_pair_kernel()
        norm = vec.norm_r(r)
        if norm <= controls.tolerance:
            converged = True
            break
        if iteration == controls.maximum_newton_iterations:
            break
        lin_tol = forcing_tolerance(norm, controls, previous_norm=prev_norm, previous_tolerance=prev_tol)
        lin_atol = 0.0 if controls.forcing_strategy == "legacy" else controls.gmres_absolute_tolerance_factor * controls.tolerance
        vec.scale_r(-1.0, r, negr)
        gm_rtol = lin_tol
        if mixed:
            sufficient = min(controls.maximum_gmres_relative_tolerance, MIXED_TARGET_SAFETY * controls.tolerance / norm)
            gm_rtol = max(lin_tol, MIXED_GMRES_FLOOR, sufficient)
        info, gm_history, gm_matvecs = solver.solve(negr, step, rtol=gm_rtol, atol=lin_atol,
                                                    maxiter=controls.gmres_maximum_restart_cycles, single=mixed,
                                                    basis_f32=mixed)
        jvp_count[0] += gm_matvecs
        if mixed:
            ops.check_device_status()
        matvec(step, jstep)
        # linear defect J s + r, merit slope r . J s, step norm
        vec.dots_r(r, 1, jstep, scal[0:1])
        defect = jstep.clone()
        vec.axpy_r(r, 1, vec.one_r, 1.0, defect)
        defect_norm = vec.norm_r(defect)
        merit_slope = float(scal[0].item())
        step_norm = vec.norm_r(step)
        true_rel = float(defect_norm / max(norm, np.finfo(float).tiny))
        if controls.forcing_strategy == "eisenstat_walker" and not _acceptable_inexact_newton_step(
                norm, merit_slope, defect_norm, relative_tolerance=lin_tol, absolute_tolerance=lin_atol):
            history.append(NewtonKrylovStep(iteration, norm, lin_tol, info, len(gm_history),
                                            tuple(gm_history), true_rel, step_norm, 0.0, norm))
            break
        damping = 1.0
        accepted_norm = np.inf
        accepted = False
        for _ in range(controls.maximum_line_search_steps):
            trial.copy_(x)
            vec.axpy_r(step, 1, vec.one_r, damping, trial)
            ops.residual(trial, jstep)
            residual_evaluations += 1
            accepted_norm = vec.norm_r(jstep)
            if accepted_norm <= (1.0 - controls.armijo * damping) * norm:
                x.copy_(trial)
                accepted = True
                if accepted_step_callback is not None:
                    amp = torch.empty(p.num_amplitudes, dtype=torch.complex128, device=dev)
                    ops.unpack(x, amp)
                    accepted_step_callback(iteration, amp.cpu().numpy(), accepted_norm)
                break
            damping *= 0.5
        history.append(NewtonKrylovStep(iteration, norm, lin_tol, info, len(gm_history),
                                        tuple(gm_history), true_rel, step_norm, float(damping), accepted_norm))
        if not accepted:
            break
        prev_norm = norm
        prev_tol = lin_tol
    jvp_evaluations = jvp_count[0]
    # independent final residual (component_solver.py:260-266)
    t0 = time.perf_counter()
    ops.residual(x, r)
    final_ref = ops.reference_value("res")
    packed = vec.norm_r(r)
    amp = torch.empty(p.num_amplitudes, dtype=torch.complex128, device=dev)
    ops.unpack(x, amp)
    rfull = torch.empty(p.num_amplitudes, dtype=torch.complex128, device=dev)
    ops.unpack(r, rfull)
    retained = rfull.cpu().numpy()
    final = ComponentStaticAction(retained, final_ref, time.perf_counter() - t0)
    return ComponentCCSolution(
        problem=p, variables=x.cpu().numpy(), amplitudes=amp.cpu().numpy(), residual=final,
        residual_norm=float(np.linalg.norm(retained)), packed_residual_norm=packed,
        reference_residual=float(abs(final_ref)), rank6=None,
        converged=bool(converged and packed <= controls.tolerance), iterations=len(history),
        residual_evaluations=residual_evaluations, jvp_evaluations=jvp_evaluations, history=tuple(history),
        preconditioner=pre, wall_seconds=float(time.perf_counter() - started),
        peak_rss_kib=int(resource.getrusage(resource.RUSAGE_SELF).ru_maxrss),
        gpu_launches=rt.LaunchCounter.count - launches0, warm_start=warm_label, device_amplitudes=amp,
    )


# Interaction scales of the reference's continuation driver
# (examples/junction/gpu_timing.py:30-31).
CONTINUATION_SCALES = (0.5, 0.75, 1.0)


@dataclass(frozen=True, slots=True)
class ContinuationStage:
    scale: float
    seconds: float
    residual: float
    iterations: int
    jvp_evaluations: int
    residual_evaluations: int


def solve_component_ccsd_continuation(problem, scales=CONTINUATION_SCALES, initial_amplitudes=None, *,
                                      policy: NewtonKrylovPolicy | None = None, precision: str = "fp64",
                                      tolerance: float = 1.0e-10):
    """Static CCSD by continuation in the interaction scale.

    The reference's production driver for strongly interacting impurities
    solves the homotopy models ``L0(K_ref) + s [L - L0(K_ref)]`` at one HF
    reference for s = 0.5, 0.75, 1, each started from the previous root, and
    stops with ``RuntimeError`` when a stage does not converge; the last scale
    is the model solved (1: the problem as compiled)
    (``examples/junction/gpu_timing.py:46-64``, problems from
    ``examples/shared/saved_reference.py:43-59``).  Returns the last stage's
    ``ComponentCCSolution`` and one ``ContinuationStage`` record per stage.
    """
    values = tuple(float(s) for s in scales)
    if not values or any(not 0.0 < s <= 1.0 for s in values) or list(values) != sorted(values):
        raise ValueError("continuation scales must increase within (0, 1]")
    initial = initial_amplitudes
    records = []
    solution = None
    for s in values:
        started = time.perf_counter()
        solution = solve_component_ccsd(problem, initial, policy=policy, precision=precision, interaction_scale=s)
        residual = solution.packed_residual_norm
        if not solution.converged or not np.isfinite(residual) or residual > tolerance:
            raise RuntimeError(f"Static solve failed at interaction scale {s}: {residual}")
        initial = solution.amplitudes
        records.append(ContinuationStage(s, time.perf_counter() - started, float(residual), solution.iterations,
                                         solution.jvp_evaluations, solution.residual_evaluations))
    return solution, tuple(records)
