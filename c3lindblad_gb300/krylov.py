"""Device Krylov solvers: restarted GMRES (Newton corrections) and CGS2 Arnoldi.

Vectors live on the GPU; every vector operation is a kernel of the C ABI.
Only O(restart) / O(m) scalars (projection coefficients, norms) cross to the
host per iteration, where the Givens updates and stopping tests run.
"""

from __future__ import annotations

import ctypes as C
import math
import time
from dataclasses import dataclass

import numpy as np
import torch

from . import runtime as rt


class DeviceVectors:
    """Thin wrappers of the library's vector kernels on one device."""

    def __init__(self, device):
        self.device = device
        self.lib = rt.lib()
        self.one_r = torch.ones(1, dtype=torch.float64, device=device)
        self.one_c = torch.ones(1, dtype=torch.complex128, device=device)
        self._partial: dict = {}

    def s(self) -> int:
        return rt.stream_ptr(self.device)

    def _scratch(self, k: int, dim: int, dtype) -> torch.Tensor:
        need = int(self.lib.c3l_multi_dot_scratch(k, dim))
        key = dtype
        buf = self._partial.get(key)
        if buf is None or buf.numel() < need:
            buf = torch.empty(max(need, 1024), dtype=dtype, device=self.device)
            self._partial[key] = buf
        return buf

    # real ------------------------------------------------------------
    def dots_r(self, V: torch.Tensor, k: int, w: torch.Tensor, out: torch.Tensor) -> None:
        dim = w.numel()
        ld = V.stride(0) if V.dim() == 2 else dim
        rt.check(self.lib.c3l_multi_dot_r(V.data_ptr(), ld, k, w.data_ptr(), dim,
                                          self._scratch(k, dim, torch.float64).data_ptr(), out.data_ptr(), self.s()),
                 "multi_dot_r")
        rt.LaunchCounter.add(2)

    def axpy_r(self, V: torch.Tensor, k: int, c: torch.Tensor, alpha: float, w: torch.Tensor) -> None:
        dim = w.numel()
        ld = V.stride(0) if V.dim() == 2 else dim
        rt.check(self.lib.c3l_multi_axpy_r(V.data_ptr(), ld, k, c.data_ptr(), float(alpha), w.data_ptr(), dim, self.s()),
                 "multi_axpy_r")
        rt.LaunchCounter.add(1)

    def scale_r(self, a: float, x: torch.Tensor, y: torch.Tensor) -> None:
        rt.check(self.lib.c3l_scale_r(x.numel(), float(a), x.data_ptr(), y.data_ptr(), self.s()), "scale_r")
        rt.LaunchCounter.add(1)

    def norm_r(self, x: torch.Tensor, out: torch.Tensor | None = None) -> float:
        buf = out if out is not None else torch.empty(1, dtype=torch.float64, device=self.device)
        self.dots_r(x, 1, x, buf)
        return math.sqrt(max(float(buf[0].item()), 0.0))

    # complex ---------------------------------------------------------
    def dots_c(self, V: torch.Tensor, k: int, w: torch.Tensor, out: torch.Tensor) -> None:
        dim = w.numel()
        ld = V.stride(0) if V.dim() == 2 else dim
        rt.check(self.lib.c3l_multi_dot_c(V.data_ptr(), ld, k, w.data_ptr(), dim,
                                          self._scratch(k, dim, torch.complex128).data_ptr(), out.data_ptr(), self.s()),
                 "multi_dot_c")
        rt.LaunchCounter.add(2)

    def axpy_c(self, V: torch.Tensor, k: int, c: torch.Tensor, alpha: complex, w: torch.Tensor) -> None:
        dim = w.numel()
        ld = V.stride(0) if V.dim() == 2 else dim
        rt.check(self.lib.c3l_multi_axpy_c(V.data_ptr(), ld, k, c.data_ptr(), rt.cplx(alpha), w.data_ptr(), dim, self.s()),
                 "multi_axpy_c")
        rt.LaunchCounter.add(1)

    def scale_c(self, a: complex, x: torch.Tensor, y: torch.Tensor) -> None:
        rt.check(self.lib.c3l_scale_c(x.numel(), rt.cplx(a), x.data_ptr(), y.data_ptr(), self.s()), "scale_c")
        rt.LaunchCounter.add(1)


# =================================================================== GMRES
def _lartg(f: float, g: float):
    """Real plane rotation with c*f + s*g = r, -s*f + c*g = 0."""
    if g == 0.0:
        return 1.0, 0.0, f
    if f == 0.0:
        return 0.0, math.copysign(1.0, g), abs(g)
    r = math.hypot(f, g)
    c = abs(f) / r
    s = math.copysign(1.0, f) * g / r
    return c, s, math.copysign(r, f)


@dataclass
class GMRESResult:
    x: torch.Tensor
    info: int
    history: list


def gmres(vec: DeviceVectors, matvec, psolve, b: torch.Tensor, *, rtol: float, atol: float, restart: int,
          maxiter: int) -> GMRESResult:
    """Left-preconditioned restarted GMRES with SciPy's control flow.

    Follows ``scipy.sparse.linalg.gmres`` (the solver the reference calls at
    ``src/c3l/cc/component_solver.py:181``): the preconditioned residual drives
    the inner loop, the true residual ``b - A x`` is checked after each
    cycle, and the inner tolerance is adapted between cycles.  Orthogonal-
    ization is classical Gram--Schmidt twice on the device.
    """
    dev = b.device
    n = b.numel()
    history: list = []
    bnrm2 = vec.norm_r(b)
    atol = max(float(atol), float(rtol) * bnrm2)
    x = torch.zeros(n, dtype=torch.float64, device=dev)
    if bnrm2 == 0.0:
        return GMRESResult(b.clone(), 0, history)
    eps = float(np.finfo(np.float64).eps)
    restart = min(restart, n)
    tmp = torch.empty(n, dtype=torch.float64, device=dev)
    psolve(b, tmp)
    Mb_nrm2 = vec.norm_r(tmp)
    ptol_max_factor = 1.0
    ptol = Mb_nrm2 * min(ptol_max_factor, atol / bnrm2)
    V = torch.empty((restart + 1, n), dtype=torch.float64, device=dev)
    coeff = torch.empty(2 * (restart + 1) + 2, dtype=torch.float64, device=dev)
    r = b.clone()
    rnorm = bnrm2
    presid = 0.0
    for iteration in range(maxiter):
        if iteration == 0 and bnrm2 < atol:
            return GMRESResult(x, 0, history)
        psolve(r, V[0])
        beta = vec.norm_r(V[0])
        vec.scale_r(1.0 / beta, V[0], V[0])
        S = np.zeros(restart + 1)
        S[0] = beta
        h = np.zeros((restart, restart + 1))
        givens = np.zeros((restart, 2))
        breakdown = False
        col = 0
        for col in range(restart):
            matvec(V[col], tmp)
            w = V[col + 1]
            psolve(tmp, w)
            k = col + 1
            c1 = coeff[:k]
            c2 = coeff[k:2 * k]
            nrm = coeff[2 * k:2 * k + 2]
            vec.dots_r(w, 1, w, nrm[0:1])               # h0^2
            vec.dots_r(V, k, w, c1)
            vec.axpy_r(V, k, c1, -1.0, w)
            vec.dots_r(V, k, w, c2)
            vec.axpy_r(V, k, c2, -1.0, w)
            vec.dots_r(w, 1, w, nrm[1:2])               # h1^2
            host = coeff[:2 * k + 2].cpu().numpy()
            h0 = math.sqrt(max(host[2 * k], 0.0))
            hcol = host[:k] + host[k:2 * k]
            h1 = math.sqrt(max(host[2 * k + 1], 0.0))
            h[col, :k] = hcol
            h[col, col + 1] = h1
            if h1 <= eps * h0:
                h[col, col + 1] = 0.0
                breakdown = True
            else:
                vec.scale_r(1.0 / h1, w, w)
            for j in range(col):
                c, s = givens[j]
                n0, n1 = h[col, j], h[col, j + 1]
                h[col, j], h[col, j + 1] = c * n0 + s * n1, -s * n0 + c * n1
            c, s, mag = _lartg(h[col, col], h[col, col + 1])
            givens[col] = (c, s)
            h[col, col], h[col, col + 1] = mag, 0.0
            t = -s * S[col]
            S[col], S[col + 1] = c * S[col], t
            presid = abs(t)
            history.append(presid / bnrm2)
            if presid <= ptol or breakdown:
                break
        if h[col, col] == 0:
            S[col] = 0
        y = np.array(S[:col + 1], dtype=np.float64)
        for j in range(col, 0, -1):
            if y[j] != 0:
                y[j] /= h[j, j]
                y[:j] -= y[j] * h[j, :j]
        if y[0] != 0:
            y[0] /= h[0, 0]
        ydev = torch.from_numpy(y).to(dev)
        vec.axpy_r(V, col + 1, ydev, 1.0, x)
        matvec(x, tmp)
        r.copy_(b)
        vec.axpy_r(tmp, 1, vec.one_r, -1.0, r)
        rnorm = vec.norm_r(r)
        if rnorm <= atol:
            break
        elif breakdown:
            break
        elif presid <= ptol:
            ptol_max_factor = max(eps, 0.25 * ptol_max_factor)
        else:
            ptol_max_factor = min(1.0, 1.5 * ptol_max_factor)
        ptol = presid * min(ptol_max_factor, atol / rnorm)
    info = 0 if rnorm <= atol else maxiter
    return GMRESResult(x, info, history)


# ================================================================= Arnoldi
@dataclass
class ArnoldiBasis:
    """Krylov basis V (rows) and Hessenberg H of K V_m = V_m H_m + h v e_m^T."""

    V: torch.Tensor          # [m+1, N] complex (device)
    H: np.ndarray            # [m+1, m] complex (host)
    beta: float
    m: int
    breakdown: bool
    check_dimensions: list
    check_residuals: list
    converged: bool
    action_seconds: float
    wall_seconds: float


def hessenberg_shifted(H: np.ndarray, m: int, shifts: torch.Tensor, beta: float, sinkproj: torch.Tensor | None):
    """Green-function values and Arnoldi residuals for all shifts (device)."""
    dev = shifts.device
    lib = rt.lib()
    Hd = torch.from_numpy(np.ascontiguousarray(H[:m + 1, :m])).to(dev)
    ns = shifts.numel()
    green = torch.empty(ns, dtype=torch.complex128, device=dev) if sinkproj is not None else None
    resid = torch.empty(ns, dtype=torch.float64, device=dev)
    rt.check(lib.c3l_hessenberg_shifted(Hd.data_ptr(), m, m, shifts.data_ptr(), ns, float(beta),
                                        rt.ptr(sinkproj), rt.ptr(green), resid.data_ptr(), rt.stream_ptr(dev)),
             "hessenberg_shifted")
    rt.LaunchCounter.add(1)
    return green, resid


def arnoldi(vec: DeviceVectors, matvec, b: torch.Tensor, shifts: torch.Tensor, *, maximum_dimension: int,
            residual_tolerance: float, minimum_dimension: int = 16, check_interval: int = 8,
            breakdown_tolerance: float = 1.0e-14) -> ArnoldiBasis:
    """Two-pass classical Gram--Schmidt Arnoldi for (z I - K)^{-1} b.

    Same recurrence, breakdown test and stopping rule as the reference's
    ``arnoldi_resolvent`` (``src/c3l/green/krylov.py:284-417``); the reduced
    shifted solves for the stopping test run on the device for all shifts.
    """
    started = time.perf_counter()
    dev = b.device
    N = b.numel()
    m_max = int(maximum_dimension)
    if m_max < 1 or m_max > N:
        raise ValueError("maximum_dimension must lie in [1, operator.dimension]")
    beta = vec.norm_r(torch.view_as_real(b).reshape(-1))
    if beta == 0.0:
        raise ValueError("rhs must be nonzero")
    V = torch.empty((m_max + 1, N), dtype=torch.complex128, device=dev)
    H = np.zeros((m_max + 1, m_max), dtype=np.complex128)
    vec.scale_c(1.0 / beta, b, V[0])
    coeff = torch.empty(2 * (m_max + 1) + 1, dtype=torch.complex128, device=dev)
    check_dims: list = []
    check_res: list = []
    actual = m_max
    breakdown = False
    action = 0.0
    for j in range(m_max):
        t0 = time.perf_counter()
        w = V[j + 1]
        matvec(V[j], w)
        action += time.perf_counter() - t0
        k = j + 1
        c1 = coeff[:k]
        c2 = coeff[k:2 * k]
        nrm = coeff[2 * k:2 * k + 1]
        vec.dots_c(V, k, w, c1)
        vec.axpy_c(V, k, c1, -1.0, w)
        vec.dots_c(V, k, w, c2)
        vec.axpy_c(V, k, c2, -1.0, w)
        vec.dots_c(w, 1, w, nrm)
        host = coeff[:2 * k + 1].cpu().numpy()
        if not np.all(np.isfinite(host)):
            raise FloatingPointError("Nonfinite Arnoldi step")
        H[:k, j] = host[:k] + host[k:2 * k]
        hn = math.sqrt(max(host[2 * k].real, 0.0))
        H[j + 1, j] = hn
        actual = j + 1
        if abs(hn) <= breakdown_tolerance:
            breakdown = True
            break
        vec.scale_c(1.0 / hn, w, w)
        if actual >= minimum_dimension and (actual % check_interval == 0 or actual == m_max):
            _, res = hessenberg_shifted(H, actual, shifts, beta, None)
            worst = float(res.max().item())
            check_dims.append(actual)
            check_res.append(worst)
            if worst <= residual_tolerance:
                break
    if not check_dims or check_dims[-1] != actual:
        _, res = hessenberg_shifted(H, actual, shifts, beta, None)
        check_dims.append(actual)
        check_res.append(float(res.max().item()))
    return ArnoldiBasis(V, H[:actual + 1, :actual], beta, actual, breakdown, check_dims, check_res,
                        bool(check_res[-1] <= residual_tolerance), action, time.perf_counter() - started)


def project_sink(vec: DeviceVectors, basis: ArnoldiBasis, sink: torch.Tensor) -> torch.Tensor:
    """p_k = sink . v_k (bilinear, no conjugation) for k < m."""
    out = torch.empty(basis.m, dtype=torch.complex128, device=sink.device)
    vec.dots_c(basis.V, basis.m, torch.conj(sink).resolve_conj().contiguous(), out)
    return torch.conj(out).resolve_conj()


def reduced_coordinates(basis: ArnoldiBasis, shifts: torch.Tensor, chunk_bytes: int = 1 << 30) -> torch.Tensor:
    """Y[s, :m] with (z_s I - H_m) y = beta e_1, via caller-held R scratch."""
    dev = shifts.device
    lib = rt.lib()
    m = basis.m
    Hd = torch.from_numpy(np.ascontiguousarray(basis.H[:m + 1, :m])).to(dev)
    ns = shifts.numel()
    per = m * (m + 1) // 2
    chunk = max(1, min(ns, chunk_bytes // max(1, per * 16)))
    scratch = torch.empty(chunk * per, dtype=torch.complex128, device=dev)
    Y = torch.empty((ns, m), dtype=torch.complex128, device=dev)
    for s0 in range(0, ns, chunk):
        s1 = min(ns, s0 + chunk)
        rt.check(lib.c3l_hessenberg_coordinates(Hd.data_ptr(), m, m, shifts[s0:s1].data_ptr(), s1 - s0,
                                                float(basis.beta), scratch.data_ptr(), Y[s0:s1].data_ptr(),
                                                rt.stream_ptr(dev)), "hessenberg_coordinates")
        rt.LaunchCounter.add(1)
    return Y
