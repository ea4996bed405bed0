"""Device-resident operators: static residual/JVP and EOM sigma.

Each operator owns a complex workspace holding padded source blocks, atoms
and rest forms, uploads its program tables once, and launches the kernel
sequence of one action through a single C-ABI call
(``c3l_static_apply`` / ``c3l_eom_sigma`` / ``c3l_action_prepare``).
"""

from __future__ import annotations

import ctypes as C
import os

import numpy as np
import torch

from . import runtime as rt
from .plans import EOMPlan, SourcePlan, StaticPlan


PAIR_KERNELS = {"simt": rt.PAIR_SIMT, "tcgen05": rt.PAIR_TCGEN05}
# the kernel used before (or without) tuning
PAIR_KERNEL_DEFAULT = "auto"


def pair_kernel_setting() -> str:
    """C3L_PAIR_KERNEL: 'simt' or 'tcgen05' forces the FP32 JVP's pair-GEMM
    kernel; 'auto' lets the first mixed-precision solve time both and keep the
    faster (``DeviceStatic.tune_pair_kernel``)."""
    v = os.environ.get("C3L_PAIR_KERNEL", PAIR_KERNEL_DEFAULT)
    return v if v in ("simt", "tcgen05", "auto") else PAIR_KERNEL_DEFAULT


def pair_kernel() -> int:
    """The kernel a new action starts with (the CUDA cores under 'auto', until
    the autotuner has timed both)."""
    v = pair_kernel_setting()
    return PAIR_KERNELS["simt" if v == "auto" else v]


def _cz(n: int, device) -> torch.Tensor:
    return torch.zeros(max(n, 1), dtype=torch.complex128, device=device)


def _preconditioner_tables(plan: StaticPlan):
    """(M blocks per representative, diagnostics, the same blocks in the JVP
    output stage's element order for the fused M J): a function of the
    compiled plan, formed once per plan."""
    cached = plan.__dict__.get("_pc_tables")
    if cached is None:
        m4, diagnostics = plan.preconditioner_table()
        t = plan.tilde
        rep_of = np.full(plan.num_amplitudes, -1, np.int64)
        rep_of[t.rep_pos] = np.arange(t.rep_pos.size)
        elem_rep = rep_of[plan.program.stages["jvp"].elements]
        if np.any(elem_rep < 0):
            raise rt.C3LError("JVP output elements must be tilde representatives")
        cached = (m4, diagnostics, np.ascontiguousarray(m4[elem_rep]))
        plan.__dict__["_pc_tables"] = cached
    return cached


class DeviceStatic:
    """Residual, linearization and exact JVP in real tilde coordinates."""

    def __init__(self, plan: StaticPlan, device=None):
        self.device = rt.require_cuda(device)
        self.lib = rt.lib()
        self.plan = plan
        prog = plan.program
        up = rt.Uploader(self.device)
        self._up = up
        self.D = plan.num_variables
        self.A = plan.num_amplitudes
        # FP64 workspaces: the workspace, then the pair buffer of the residual's output
        # stage (double-float pair GEMMs)
        self.ws_lin = _cz(prog.ws_size + prog.pair_size, self.device)
        self.ws_res = _cz(prog.ws_size + prog.pair_size, self.device)
        with up.batch():  # every table of the static actions in one copy per arena chunk (no launch inside)
            vec = up.raw(prog.vectors)
            self.vec = vec
            t = plan.tilde
            ia, ib = up.raw(t.idx_a), up.raw(t.idx_b)
            ca, cb = up.raw(t.coef_a), up.raw(t.coef_b)
            self.canon_T = _cz(self.A, self.device)
            self.canon_R = _cz(self.A, self.device)
            self.canon_V = _cz(self.A, self.device)

            self.pair_status = torch.zeros(1, dtype=torch.int32, device=self.device)

            def static_action(ws, levels_cls, padded, out, scatter, canon, ep, vectors=vec, pairs=None, kernel=0):
                sa = rt.StaticAction()
                sa.action = rt.build_action(up, prog, vectors.data_ptr(), ws, levels_cls, padded, out, scatter, pairs,
                                            kernel, self.pair_status.data_ptr())
                sa.num_amplitudes = self.A
                sa.tilde_ia, sa.tilde_ib = ia.data_ptr(), ib.data_ptr()
                sa.tilde_ca, sa.tilde_cb = ca.data_ptr(), cb.data_ptr()
                sa.canon = canon.data_ptr()
                sa.lam = up.ptr(ep["lam"])
                sa.col = up.ptr(ep["col"])
                sa.pair = up.ptr(ep["pair"])
                sa.scale = up.ptr(ep["scale"])
                sa.interaction_scale = 1.0
                return sa

            rp = "res" if "res" in prog.pairs else None
            self.res_action = static_action(self.ws_res, "T", ["res_rest_T", "res_scalar"],
                                            "res_pairs" if rp else "res", plan.scatter_T, self.canon_R, plan.epilogue,
                                            pairs=rp)
            self.lin_action = static_action(self.ws_lin, "T", ["res_rest_T", "res_scalar", "jvp_rest_T"],
                                            "res_pairs" if rp else "res", plan.scatter_T, self.canon_T, plan.epilogue,
                                            pairs=rp)
            jp = "jvp" if "jvp" in prog.pairs else None
            self.jvp_action = static_action(self.ws_lin, "V", ["jvp_rest_V", "jvp_scalar"],
                                            "jvp_pairs" if jp else "jvp", plan.scatter_V, self.canon_V,
                                            plan.epilogue_jvp, pairs=jp)
            # single-precision twin of the JVP (inner operator of the mixed-precision solve):
            # its output stage sums the anchor ^ rest products as pair GEMMs into the
            # pair buffer that follows the FP32 workspace, then gathers them
            self.vec32 = up.raw(prog.vectors.astype(np.complex64))
            self.ws32_lin = torch.zeros(max(prog.ws_size + prog.pair_size, 1), dtype=torch.complex64,
                                        device=self.device)
            pairs = "jvp" if "jvp" in prog.pairs else None
            self.pair_kernel = pair_kernel()
            self.pair_tuning = None  # {kernel: ms} once tuned
            self.jvp32_action = static_action(self.ws32_lin, "V", ["jvp_rest_V", "jvp_scalar"],
                                              "jvp_pairs" if pairs else "jvp", plan.scatter_V, self.canon_V,
                                              plan.epilogue_jvp, vectors=self.vec32, pairs=pairs,
                                              kernel=self.pair_kernel)
            # complex outputs at every coordinate (arbitrary complex amplitudes)
            self.cres_action = rt.build_action(up, prog, vec.data_ptr(), self.ws_res, "T", ["res_rest_T", "res_scalar"],
                                               None, plan.scatter_T)
            self.cres_stage = rt.wedge_stage(up, prog.stages["res_all"])
            self.cres_lam = up.raw(plan.lam_all)
            self.clin_action = rt.build_action(up, prog, vec.data_ptr(), self.ws_lin, "T", ["jvp_rest_T"], None,
                                               plan.scatter_T)
            self.cjvp_action = rt.build_action(up, prog, vec.data_ptr(), self.ws_lin, "V", ["jvp_rest_V", "jvp_scalar"],
                                               None, plan.scatter_V)
            self.cjvp_stage = rt.wedge_stage(up, prog.stages["jvp_all"])
            self.cjvp_lam = up.raw(plan.lam_all_jvp)
            self.launches = {
                "residual": rt.static_launches(self.res_action.action),
                "linearize": rt.static_launches(self.lin_action.action),
                "jvp": rt.static_launches(self.jvp_action.action),
                "jvp32": rt.static_launches(self.jvp32_action.action),
            }
            m4, self.preconditioner_diagnostics, m4_elem = _preconditioner_tables(plan)
            self.pc_m4 = up.raw(m4)
            self.pc_col = up.raw(t.rep_col)
            self.pc_pair = up.raw(t.rep_pair)
            self.pc_m4_elem = up.raw(m4_elem)
            self.nrep = int(t.rep_pos.size)
            self.ia, self.ib, self.ca, self.cb = ia, ib, ca, cb

    def _stream(self) -> int:
        return rt.stream_ptr(self.device)

    @property
    def interaction_scale(self) -> float:
        return float(self.res_action.interaction_scale)

    def set_interaction_scale(self, s: float) -> None:
        """Scale the product part of the residual and JVP (the homotopy
        ``L0(K_ref) + s [L - L0(K_ref)]`` at the compiled HF reference)."""
        s = float(s)
        if not 0.0 <= s <= 1.0:
            raise ValueError("interaction scale must lie in [0, 1]")
        for a in (self.res_action, self.lin_action, self.jvp_action, self.jvp32_action):
            a.interaction_scale = s

    def _apply(self, action, x: torch.Tensor, out: torch.Tensor, what: str, launches: int) -> None:
        if x.dtype != torch.float64 or out.dtype != torch.float64 or x.numel() != self.D or out.numel() != self.D:
            raise ValueError(f"{what}: expected float64 vectors of length {self.D}")
        rt.check(self.lib.c3l_static_apply(C.byref(action), x.data_ptr(), out.data_ptr(), self._stream()), what)
        rt.LaunchCounter.add(launches)

    def residual(self, x: torch.Tensor, out: torch.Tensor) -> None:
        """Real residual at x (independent of the linearization point)."""
        self._apply(self.res_action, x, out, "static residual", self.launches["residual"])

    def linearize(self, x: torch.Tensor, out: torch.Tensor) -> None:
        """Residual at x; also caches the amplitude-only JVP data at x."""
        self._apply(self.lin_action, x, out, "static linearization", self.launches["linearize"])

    def jvp(self, v: torch.Tensor, out: torch.Tensor) -> None:
        """Exact JVP at the last linearization point."""
        self._apply(self.jvp_action, v, out, "static JVP", self.launches["jvp"])

    def to_single(self) -> None:
        """Copy the linearization workspace into its FP32 twin (after ``linearize``)."""
        rt.check(self.lib.c3l_downcast(self.plan.program.ws_size, self.ws_lin.data_ptr(), self.ws32_lin.data_ptr(),
                                       self._stream()), "downcast")
        rt.LaunchCounter.add(1)

    def jvp32(self, v: torch.Tensor, out: torch.Tensor) -> None:
        """JVP with FP32 contractions at the last linearization point (after ``to_single``)."""
        if v.dtype != torch.float64 or out.dtype != torch.float64 or v.numel() != self.D or out.numel() != self.D:
            raise ValueError(f"jvp32: expected float64 vectors of length {self.D}")
        rt.check(self.lib.c3l_static_apply_f32(C.byref(self.jvp32_action), v.data_ptr(), out.data_ptr(),
                                               self._stream()), "static JVP (fp32)")
        rt.LaunchCounter.add(self.launches["jvp32"])

    @property
    def pair_kernel_name(self) -> str:
        return {v: k for k, v in PAIR_KERNELS.items()}[int(self.jvp32_action.action.pairs.kernel)]

    def tune_pair_kernel(self, reps: int = 3) -> dict:
        """Project autotuner of the FP32 JVP's contraction tiles: times the JVP
        (after ``to_single``) with each pair-GEMM kernel -- CUDA cores on the
        compiler's per-group tile shapes, tcgen05 tensor cores on 128 x 64
        tiles -- and keeps the faster.
        Returns {kernel: milliseconds}.  Both kernels sum in FP32 (the
        tensor-core one in split TF32), so the choice does not move the JVP
        beyond FP32 rounding."""
        if self.jvp32_action.action.pairs.ntiles <= 0:
            return {}
        times = {}
        v = torch.zeros(self.D, dtype=torch.float64, device=self.device)
        v[:: max(self.D // 97, 1)] = 1.0
        out = torch.empty_like(v)
        for name, k in PAIR_KERNELS.items():
            self.jvp32_action.action.pairs.kernel = k
            self.jvp32(v, out)  # first launch: function attributes, caches
            torch.cuda.synchronize(self.device)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(reps):
                self.jvp32(v, out)
            e1.record()
            torch.cuda.synchronize(self.device)
            self.check_device_status()
            times[name] = e0.elapsed_time(e1) / reps
        best = min(times, key=times.get)
        self.jvp32_action.action.pairs.kernel = PAIR_KERNELS[best]
        self.pair_tuning = times
        return times

    def check_device_status(self) -> None:
        """Raise if a tensor-core pair GEMM block gave up waiting for its MMAs."""
        if int(self.pair_status.item()) != 0:
            self.pair_status.zero_()
            raise rt.C3LError("a tensor-core pair GEMM timed out waiting for its MMAs")

    def precondition(self, x: torch.Tensor, out: torch.Tensor) -> None:
        rt.check(self.lib.c3l_precondition(self.nrep, self.pc_m4.data_ptr(), self.pc_col.data_ptr(),
                                           self.pc_pair.data_ptr(), x.data_ptr(), out.data_ptr(), self._stream()),
                 "preconditioner")
        rt.LaunchCounter.add(1)

    def unpack(self, x: torch.Tensor, out: torch.Tensor) -> None:
        """Complex amplitudes (reference vector order) from real variables."""
        rt.check(self.lib.c3l_tilde_unpack(self.A, x.data_ptr(), self.ia.data_ptr(), self.ib.data_ptr(),
                                           self.ca.data_ptr(), self.cb.data_ptr(), out.data_ptr(), self._stream()),
                 "tilde unpack")
        rt.LaunchCounter.add(1)

    def reference_value(self, which: str = "res") -> complex:
        off = self.plan.res_scalar_off
        ws = self.ws_res if which == "res" else self.ws_lin
        if off < 0:
            return 0j
        return complex(-1j * self.interaction_scale * ws[off].item())

    # ---------------------------------------------- complex-amplitude actions
    def residual_complex(self, t: torch.Tensor, out: torch.Tensor) -> complex:
        """-i pack(Lambda T + V) at all coordinates for arbitrary complex amplitudes."""
        s = self._stream()
        rt.check(self.lib.c3l_action_prepare(C.byref(self.cres_action), t.data_ptr(), s), "residual prepare")
        rt.check(self.lib.c3l_wedge_eom_out(C.byref(self.cres_stage), self.plan.n, self.ws_res.data_ptr(),
                                            self.cres_lam.data_ptr(), t.data_ptr(), out.data_ptr(), s), "residual out")
        rt.LaunchCounter.add(rt.action_launches(self.cres_action) + 1)
        return self.reference_value("res")

    def jvp_complex(self, t: torch.Tensor, v: torch.Tensor, out: torch.Tensor) -> complex:
        s = self._stream()
        rt.check(self.lib.c3l_action_prepare(C.byref(self.clin_action), t.data_ptr(), s), "jvp linearize")
        rt.check(self.lib.c3l_action_prepare(C.byref(self.cjvp_action), v.data_ptr(), s), "jvp prepare")
        rt.check(self.lib.c3l_wedge_eom_out(C.byref(self.cjvp_stage), self.plan.n, self.ws_lin.data_ptr(),
                                            self.cjvp_lam.data_ptr(), v.data_ptr(), out.data_ptr(), s), "jvp out")
        rt.LaunchCounter.add(rt.action_launches(self.clin_action) + rt.action_launches(self.cjvp_action) + 1)
        off = self.plan.jvp_scalar_off
        return 0j if off < 0 else complex(-1j * self.ws_lin[off].item())


class DeviceEOM:
    """Sigma action of one (spin, charge) EOM block at fixed amplitudes."""

    def __init__(self, plan: EOMPlan, amplitudes: torch.Tensor, device=None, tables: dict | None = None,
                 interaction_scale: float = 1.0):
        """``tables``: a dict (device -> Uploader) owned by the EOM problem, so that
        contexts of one problem share its uploaded program tables.
        ``interaction_scale``: the product part's factor (the homotopy model
        the amplitudes were solved at)."""
        if not 0.0 <= float(interaction_scale) <= 1.0:
            raise ValueError("interaction scale must lie in [0, 1]")
        self.interaction_scale = float(interaction_scale)
        self.device = rt.require_cuda(device)
        self.lib = rt.lib()
        self.plan = plan
        prog = plan.program
        if tables is None:
            tables = {}
        up = tables.get(self.device)
        if up is None:
            up = tables[self.device] = rt.Uploader(self.device)
        self._up = up
        self.N = plan.dimension
        with up.batch():
            self.vec = up.table(prog.vectors)
            self.lam = up.table(plan.lam_sigma)
        self.amplitudes = amplitudes.to(self.device, torch.complex128).contiguous()
        self.workspaces: list = []
        self.sigma_actions: list = []
        self.ensure_channels(1)
        self.ws = self.workspaces[0]
        self.sigma_action = self.sigma_actions[0]
        self.sigma_launches = rt.action_launches(self.sigma_action.action)
        self.diagonal = torch.from_numpy(plan.diagonal.copy()).to(self.device)

    def input_scatter_csr(self):
        """(offsets[N+1], dst, sign) device tables: the nonzero entries of the
        sigma's input scatter grouped by input element (uploaded once)."""
        csr = self.plan.__dict__.get("_x_scatter_csr")
        if csr is None:
            sc = self.plan.scatter_X
            keep = np.nonzero(sc.sign != 0.0)[0]
            order = keep[np.argsort(sc.pos[keep], kind="stable")]
            offsets = np.zeros(self.N + 1, dtype=np.int64)
            np.add.at(offsets, sc.pos[order] + 1, 1)
            csr = (np.cumsum(offsets), sc.dst[order].astype(np.int64), sc.sign[order].astype(np.float64))
            self.plan.__dict__["_x_scatter_csr"] = csr
        return tuple(self._up.table(a) for a in csr)

    def ensure_channels(self, count: int) -> None:
        """One workspace (amplitude part prepared) per concurrently used channel."""
        prog = self.plan.program
        up = self._up
        built = []
        pairs = "sigma" if "sigma" in prog.pairs else None
        with up.batch():  # tables sent when the block ends, before the context launches below
            while len(self.workspaces) + len(built) < count:
                # the workspace, then (pair GEMMs) the pair buffer the output stage reads
                ws = _cz(prog.ws_size + (prog.pair_size if pairs else 0), self.device)
                ctx = rt.build_action(up, prog, self.vec.data_ptr(), ws, "T", ["sigma_rest_T"], None,
                                      self.plan.scatter_T)
                ea = rt.EomAction()
                ea.action = rt.build_action(up, prog, self.vec.data_ptr(), ws, "X", ["sigma_rest_X"],
                                            "sigma_pairs" if pairs else "sigma", self.plan.scatter_X, pairs)
                ea.lam = self.lam.data_ptr()
                ea.interaction_scale = self.interaction_scale
                built.append((ws, ctx, ea))
        for ws, ctx, ea in built:
            rt.check(self.lib.c3l_action_prepare(C.byref(ctx), self.amplitudes.data_ptr(), rt.stream_ptr(self.device)),
                     "EOM context")
            rt.LaunchCounter.add(rt.action_launches(ctx))
            self.workspaces.append(ws)
            self.sigma_actions.append(ea)

    def sigma(self, x: torch.Tensor, out: torch.Tensor) -> None:
        if x.dtype != torch.complex128 or out.dtype != torch.complex128 or x.numel() != self.N:
            raise ValueError("sigma expects complex128 vectors of the EOM dimension")
        rt.check(self.lib.c3l_eom_sigma(C.byref(self.sigma_action), x.data_ptr(), out.data_ptr(),
                                        rt.stream_ptr(self.device)), "EOM sigma")
        rt.LaunchCounter.add(self.sigma_launches)

    def sources(self, site: int):
        """(addition, removal, sink) device vectors for one site."""
        sp: SourcePlan = self.plan.sources(site)
        prog = sp.program
        up = self._up
        ws = _cz(prog.ws_size, self.device)
        with up.batch():  # tables sent when the block ends, before the launches below
            vec = up.raw(prog.vectors)
            act = rt.build_action(up, prog, vec.data_ptr(), ws, "T", ["add_rest_T", "rem_rest_T"], None,
                                  sp.scatter_T)
            stages = [rt.wedge_stage(up, prog.stages.get(nm)) for nm in ("add", "rem")]
        s = rt.stream_ptr(self.device)
        rt.check(self.lib.c3l_action_prepare(C.byref(act), self.amplitudes.data_ptr(), s), "EOM source context")
        rt.LaunchCounter.add(rt.action_launches(act))
        outs = []
        for st, scale in zip(stages, sp.source_scale[:2]):
            out = _cz(self.N, self.device)
            rt.check(self.lib.c3l_wedge_source_out(C.byref(st), prog.n, ws.data_ptr(), rt.cplx(scale), out.data_ptr(), s),
                     "EOM source")
            rt.LaunchCounter.add(1)
            outs.append(out)
        sink = torch.from_numpy(sp.sink.copy()).to(self.device)
        return outs[0], outs[1], sink
