"""Device Krylov solvers: restarted GMRES (Newton corrections) and CGS2 Arnoldi.

The iteration loops run in C++ inside the library (``c3l_gmres``,
``c3l_arnoldi``); this module owns their device/pinned buffers and wraps the
vector kernels used elsewhere.  Only O(restart) / O(m) scalars cross to the
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


# ================================================================= Arnoldi
@dataclass
class ArnoldiBasis:
    """Krylov basis V (rows) and Hessenberg H of K V_m = V_m H_m + h v e_m^T.

    H stays on the device (``Hcol``: column j in row j) until it is first read."""

    V: torch.Tensor          # [m+1, N] complex (device)
    Hcol: torch.Tensor       # [m_max, m_max+1] complex (device): Hcol[j, :j+2] = H[:j+2, j]
    beta: float
    m: int
    breakdown: bool
    check_dimensions: list
    check_residuals: list
    converged: bool
    action_seconds: float
    wall_seconds: float
    green: torch.Tensor | None = None     # [nshift] sink . y at dimension m (device)
    residual: torch.Tensor | None = None  # [nshift] Arnoldi-relation residuals at m (device)
    _H: np.ndarray | None = None

    @property
    def H(self) -> np.ndarray:
        """[m+1, m] complex Hessenberg matrix (host copy, made on first use)."""
        if self._H is None:
            m = self.m
            self._H = np.ascontiguousarray(self.Hcol[:m, :m + 1].cpu().numpy().T)
        return self._H


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


def project_sink(vec: DeviceVectors, basis: ArnoldiBasis, sink: torch.Tensor) -> torch.Tensor:
    """p_k = sink . v_k (bilinear, no conjugation) for k < m."""
    out = torch.empty(basis.m, dtype=torch.complex128, device=sink.device)
    vec.dots_c(basis.V, basis.m, torch.conj(sink).resolve_conj().contiguous(), out)
    return torch.conj(out).resolve_conj()


def reduced_coordinates(basis: ArnoldiBasis, shifts: torch.Tensor, chunk_bytes: int = 1 << 30) -> torch.Tensor:
    """Y[s, :m] with (z_s I - H_m) y = beta e_1, via caller-held R scratch."""
    return hessenberg_coordinates(basis.H, basis.m, basis.beta, shifts, chunk_bytes)


def hessenberg_coordinates(H: np.ndarray, m: int, beta: float, shifts: torch.Tensor,
                           chunk_bytes: int = 1 << 30) -> torch.Tensor:
    """Y[s, :m] with (z_s I - H[:m, :m]) y = beta e_1 (device), for a host Hessenberg H[:m+1, :m]."""
    dev = shifts.device
    lib = rt.lib()
    Hd = torch.from_numpy(np.ascontiguousarray(H[:m + 1, :m])).to(dev)
    ns = shifts.numel()
    per = m * (m + 1) // 2
    chunk = max(1, min(ns, chunk_bytes // max(1, per * 16)))
    scratch = torch.empty(chunk * per, dtype=torch.complex128, device=dev)
    Y = torch.empty((ns, m), dtype=torch.complex128, device=dev)
    for s0 in range(0, ns, chunk):
        s1 = min(ns, s0 + chunk)
        rt.check(lib.c3l_hessenberg_coordinates(Hd.data_ptr(), m, m, shifts[s0:s1].data_ptr(), s1 - s0,
                                                float(beta), scratch.data_ptr(), Y[s0:s1].data_ptr(),
                                                rt.stream_ptr(dev)), "hessenberg_coordinates")
        rt.LaunchCounter.add(1)
    return Y


# ============================================================ C++ drivers
class DeviceGMRES:
    """Buffers and call wrapper for ``c3l_gmres`` (one per static problem)."""

    def __init__(self, ops, restart: int):
        self.ops = ops
        dev = ops.device
        n = ops.D
        self.restart = int(min(restart, n))
        r = self.restart
        lib = rt.lib()
        self._basis: dict = {}  # basis_f32 -> the basis buffer (allocated on first use)
        self.tmp = torch.empty(n, dtype=torch.float64, device=dev)
        self.r = torch.empty(n, dtype=torch.float64, device=dev)
        self.coeff = torch.zeros(2 * (r + 2) + 4, dtype=torch.float64, device=dev)
        self.partial = torch.empty(max(int(lib.c3l_multi_dot_scratch(r + 1, n)), int(lib.c3l_gmres_scratch(r, n)), 1),
                                   dtype=torch.float64, device=dev)
        self.host = torch.zeros(3 * (r + 2) + 4, dtype=torch.float64).pin_memory()
        self.work = torch.empty(2 * n, dtype=torch.float64, device=dev)
        self.counters = torch.zeros(4, dtype=torch.int32, device=dev)
        self.slots = torch.zeros(r * (r + 3) + 1, dtype=torch.float64).pin_memory()  # written by the GPU
        self.history = np.zeros(4096, dtype=np.float64)
        self._graphs: dict = {}  # precision -> kept inner-iteration graphs
        self._lib = lib

    def __del__(self):
        self.release_graphs()

    def release_graphs(self) -> None:
        for key, handle in list(getattr(self, "_graphs", {}).items()):
            if handle:
                self._lib.c3l_gmres_release(handle)
            self._graphs[key] = None

    def basis(self, basis_f32: bool) -> torch.Tensor:
        """The Krylov basis: restart + 1 rows of FP64, or (FP32 basis) restart + 1
        FP32 rows plus the FP32 work vector.  Only the precision in use is held."""
        got = self._basis.get(basis_f32)
        if got is None:
            r, n = self.restart, self.ops.D
            for key in list(self._basis):  # the other precision's basis and the graphs that point at it
                self.release_graphs()
                del self._basis[key]
            doubles = ((r + 2) * n + 1) // 2 if basis_f32 else (r + 1) * n
            got = torch.empty(doubles, dtype=torch.float64, device=self.ops.device)
            self._basis[basis_f32] = got
        return got

    @property
    def nbytes(self) -> int:
        return sum(t.numel() * t.element_size() for t in self._basis.values())

    def solve(self, b: torch.Tensor, x: torch.Tensor, *, rtol: float, atol: float, maxiter: int,
              single: bool = False, basis_f32: bool = False):
        """One Newton correction solve; ``single`` applies the FP32 JVP, and
        ``basis_f32`` (with ``single``) also keeps the Krylov basis in FP32."""
        ops = self.ops
        a = rt.GmresArgs()
        a.jvp = C.addressof(ops.jvp32_action if single else ops.jvp_action)
        a.use_f32 = 1 if single else 0
        a.basis_f32 = 1 if (single and basis_f32) else 0
        a.nrep = ops.nrep
        a.pc_m4, a.pc_col, a.pc_pair = ops.pc_m4.data_ptr(), ops.pc_col.data_ptr(), ops.pc_pair.data_ptr()
        a.dim = ops.D
        a.b, a.x = b.data_ptr(), x.data_ptr()
        a.rtol, a.atol = float(rtol), float(atol)
        a.restart, a.maxiter = self.restart, int(maxiter)
        a.V, a.tmp, a.r = self.basis(bool(a.basis_f32)).data_ptr(), self.tmp.data_ptr(), self.r.data_ptr()
        a.coeff, a.partial, a.host = self.coeff.data_ptr(), self.partial.data_ptr(), self.host.data_ptr()
        a.history = self.history.ctypes.data
        a.history_capacity = self.history.size
        a.work, a.counters, a.slots = self.work.data_ptr(), self.counters.data_ptr(), self.slots.data_ptr()
        a.pc_m4_elem = ops.pc_m4_elem.data_ptr()
        a.partial_capacity = self.partial.numel()
        a.keep_graphs = 1
        key = (single, bool(a.basis_f32))
        a.graph_cache = self._graphs.get(key)
        st = rt.lib().c3l_gmres(C.byref(a), rt.stream_ptr(ops.device))
        self._graphs[key] = a.graph_cache  # the call replaces a stale cache itself
        rt.check(st, "gmres")
        hist = list(self.history[:min(a.history_len, self.history.size)])
        rt.LaunchCounter.add(int(a.launches))
        return int(a.info), hist, int(a.matvecs)


class HessenbergTracker:
    """Device buffers of the incremental shifted solves of one Arnoldi basis."""

    def __init__(self, m_max: int, shifts: torch.Tensor, with_sink: bool):
        dev = shifts.device
        ns = shifts.numel()
        self.shifts = shifts
        self.rot_c = torch.empty((m_max, ns), dtype=torch.float64, device=dev)
        self.rot_s = torch.empty((m_max, ns), dtype=torch.complex128, device=dev)
        self.vsink = torch.empty((m_max, ns), dtype=torch.complex128, device=dev)
        self.carry = torch.empty(ns, dtype=torch.complex128, device=dev)
        self.accum = torch.empty(ns, dtype=torch.complex128, device=dev)
        self.green = torch.empty(ns, dtype=torch.complex128, device=dev) if with_sink else None
        self.residual = torch.empty(ns, dtype=torch.float64, device=dev)
        self.sinkproj_conj = torch.zeros(m_max, dtype=torch.complex128, device=dev) if with_sink else None
        self.status = torch.zeros(2, dtype=torch.int64, device=dev)  # c3l_hessenberg_status (16 bytes)
        self.status_host = torch.zeros(2, dtype=torch.int64).pin_memory()
        self.m_max = m_max

    def fill(self, st: rt.HessenbergState) -> None:
        st.m_max, st.nshift, st.done = self.m_max, self.shifts.numel(), 0
        st.shifts = self.shifts.data_ptr()
        st.sinkproj_conj = rt.ptr(self.sinkproj_conj)
        st.rot_c, st.rot_s, st.vsink = self.rot_c.data_ptr(), self.rot_s.data_ptr(), self.vsink.data_ptr()
        st.carry, st.accum = self.carry.data_ptr(), self.accum.data_ptr()
        st.green, st.residual, st.status = rt.ptr(self.green), self.residual.data_ptr(), self.status.data_ptr()


def arnoldi_channels(ops, sources, shifts: torch.Tensor, *, maximum_dimension: int, residual_tolerance: float,
                     minimum_dimension: int = 16, check_interval: int = 8, breakdown_tolerance: float = 1.0e-14,
                     sink: torch.Tensor | None = None):
    """Run ``c3l_arnoldi`` on several sources at once (one stream and workspace each).

    With ``sink`` the bases also carry the Green function sink . (z - K)^{-1} b
    for every shift at their final dimension (``ArnoldiBasis.green``)."""
    started = time.perf_counter()
    dev = shifts.device
    lib = rt.lib()
    N = ops.N
    m_max = int(maximum_dimension)
    nch = len(sources)
    ops.ensure_channels(nch)
    chans = (rt.ArnoldiChannel * nch)()
    streams = [torch.cuda.Stream(device=dev) for _ in range(nch)]
    cur = torch.cuda.current_stream(dev)
    sink_conj = torch.conj(sink).resolve_conj().contiguous() if sink is not None else None
    xcsr = ops.input_scatter_csr()
    per = []
    for c, b in enumerate(sources):
        d = {
            "V": torch.empty((m_max + 1, N), dtype=torch.complex128, device=dev),
            "Hcol": torch.zeros((m_max, m_max + 1), dtype=torch.complex128, device=dev),
            "coeff": torch.zeros(2 * (m_max + 1) + 2, dtype=torch.complex128, device=dev),
            "partial": torch.empty(max(int(lib.c3l_multi_dot_scratch(m_max + 1, N)), 1), dtype=torch.complex128,
                                   device=dev),
            "host": torch.zeros(2 * (m_max + 1) + 2, dtype=torch.complex128).pin_memory(),
            "cdims": np.zeros(m_max // max(check_interval, 1) + 4, dtype=np.int32),
            "hess": HessenbergTracker(m_max, shifts, sink is not None),
            "work": torch.empty(2 * N, dtype=torch.complex128, device=dev),
            "counters": torch.zeros(4, dtype=torch.int32, device=dev),
            "V32": torch.empty((m_max + 1, N), dtype=torch.complex64, device=dev),
            "work32": torch.empty(N, dtype=torch.complex64, device=dev),
            "V32lo": torch.empty((m_max + 1, N), dtype=torch.complex64, device=dev),
            "work32lo": torch.empty(N, dtype=torch.complex64, device=dev),
            "b": b,
        }
        d["cres"] = np.zeros(d["cdims"].size, dtype=np.float64)
        per.append(d)
        q = chans[c]
        q.sigma = C.addressof(ops.sigma_actions[c])
        q.b, q.sink_conj = b.data_ptr(), rt.ptr(sink_conj)
        q.V, q.Hcol, q.coeff = d["V"].data_ptr(), d["Hcol"].data_ptr(), d["coeff"].data_ptr()
        q.partial, q.host, q.H = d["partial"].data_ptr(), d["host"].data_ptr(), None  # H stays on the device
        d["hess"].fill(q.hess)
        q.status_host = d["hess"].status_host.data_ptr()
        q.work, q.counters = d["work"].data_ptr(), d["counters"].data_ptr()
        q.V32, q.work32 = d["V32"].data_ptr(), d["work32"].data_ptr()
        q.V32lo, q.work32lo = d["V32lo"].data_ptr(), d["work32lo"].data_ptr()
        q.xscatter_offsets, q.xscatter_dst, q.xscatter_sign = (t.data_ptr() for t in xcsr)
        q.check_dims, q.check_res, q.check_capacity = d["cdims"].ctypes.data, d["cres"].ctypes.data, d["cdims"].size
    for st in streams:
        st.wait_stream(cur)
    sp = (C.c_void_p * nch)(*[st.cuda_stream for st in streams])
    rt.check(lib.c3l_arnoldi(chans, nch, N, shifts.data_ptr(), shifts.numel(), m_max, float(residual_tolerance),
                             int(minimum_dimension), int(check_interval), float(breakdown_tolerance), sp), "arnoldi")
    for st in streams:
        cur.wait_stream(st)
    out = []
    for c in range(nch):
        q = chans[c]
        d = per[c]
        m = int(q.m)
        nchk = min(int(q.nchecks), d["cdims"].size)
        rt.LaunchCounter.add(int(q.launches))
        out.append(ArnoldiBasis(d["V"], d["Hcol"], float(q.beta), m, bool(q.breakdown),
                                list(d["cdims"][:nchk]), list(d["cres"][:nchk]), bool(q.converged),
                                float(q.action_seconds), time.perf_counter() - started,
                                d["hess"].green, d["hess"].residual))
    return out
