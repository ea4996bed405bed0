"""ctypes binding of ``libc3l_gb300.so`` and device-resident plan state.

PyTorch provides device memory and the current CUDA stream; every kernel is
launched through the library's C ABI (``include/c3l_gb300.h``).  Nothing here
computes on the host: when the library or a GPU is missing the calls raise.
"""

from __future__ import annotations

import contextlib
import ctypes as C
from pathlib import Path

import numpy as np
import torch

from . import _build

_LIB = None


class C3LError(RuntimeError):
    pass


# ----------------------------------------------------------------- structs
class ContractLevel(C.Structure):
    _fields_ = [("tasks", C.c_void_p), ("tiles", C.c_void_p), ("ntiles", C.c_int64)]


class PairProgram(C.Structure):
    _fields_ = [("groups", C.c_void_p), ("aoff", C.c_void_p), ("roff", C.c_void_p), ("tiles", C.c_void_p),
                ("ntiles", C.c_int64), ("base", C.c_int64), ("tiles_tc", C.c_void_p), ("ntiles_tc", C.c_int64),
                ("status", C.c_void_p), ("kernel", C.c_int32), ("pad", C.c_int32)]


PAIR_SIMT, PAIR_TCGEN05 = 0, 1


class WedgeStage(C.Structure):
    _fields_ = [("blocks", C.c_void_p), ("instances", C.c_void_p), ("tiles", C.c_void_p),
                ("ntiles", C.c_int64), ("elements", C.c_void_p), ("digits", C.c_void_p), ("width", C.c_int32),
                ("pad", C.c_int32)]


class Action(C.Structure):
    _fields_ = [("n", C.c_int32), ("nlevels", C.c_int32), ("npadded", C.c_int32), ("pad", C.c_int32),
                ("vectors", C.c_void_p), ("ws", C.c_void_p), ("scatter_count", C.c_int64),
                ("scatter_dst", C.c_void_p), ("scatter_pos", C.c_void_p), ("scatter_sign", C.c_void_p),
                ("levels", ContractLevel * 8), ("padded", WedgeStage * 4), ("pairs", PairProgram),
                ("out", WedgeStage)]


class StaticAction(C.Structure):
    _fields_ = [("action", Action), ("num_amplitudes", C.c_int64), ("tilde_ia", C.c_void_p),
                ("tilde_ib", C.c_void_p), ("tilde_ca", C.c_void_p), ("tilde_cb", C.c_void_p),
                ("canon", C.c_void_p), ("lam", C.c_void_p), ("col", C.c_void_p), ("pair", C.c_void_p),
                ("scale", C.c_void_p), ("pc_m4", C.c_void_p), ("interaction_scale", C.c_double)]


class EomAction(C.Structure):
    _fields_ = [("action", Action), ("lam", C.c_void_p), ("interaction_scale", C.c_double)]


class Complex(C.Structure):
    _fields_ = [("re", C.c_double), ("im", C.c_double)]


class GmresArgs(C.Structure):
    _fields_ = [("jvp", C.c_void_p), ("nrep", C.c_int64), ("pc_m4", C.c_void_p), ("pc_col", C.c_void_p),
                ("pc_pair", C.c_void_p), ("dim", C.c_int64), ("b", C.c_void_p), ("x", C.c_void_p),
                ("rtol", C.c_double), ("atol", C.c_double), ("restart", C.c_int32), ("maxiter", C.c_int32),
                ("V", C.c_void_p), ("tmp", C.c_void_p), ("r", C.c_void_p), ("coeff", C.c_void_p),
                ("partial", C.c_void_p), ("host", C.c_void_p), ("history", C.c_void_p),
                ("history_capacity", C.c_int32), ("history_len", C.c_int32), ("info", C.c_int32),
                ("matvecs", C.c_int32), ("use_f32", C.c_int32), ("work", C.c_void_p), ("counters", C.c_void_p),
                ("slots", C.c_void_p), ("launches", C.c_int64), ("pc_m4_elem", C.c_void_p),
                ("partial_capacity", C.c_int64), ("keep_graphs", C.c_int32), ("basis_f32", C.c_int32),
                ("graph_cache", C.c_void_p)]


class GmresShiftedArgs(C.Structure):
    _fields_ = [("sigma", C.c_void_p), ("sigma_launches", C.c_int32), ("use_x0", C.c_int32), ("dim", C.c_int64),
                ("shift", Complex), ("pc_inv", C.c_void_p), ("b", C.c_void_p), ("x", C.c_void_p),
                ("rtol", C.c_double), ("atol", C.c_double), ("restart", C.c_int32), ("maxiter", C.c_int32),
                ("V", C.c_void_p), ("tmp", C.c_void_p), ("r", C.c_void_p), ("coeff", C.c_void_p),
                ("partial", C.c_void_p), ("host", C.c_void_p), ("history", C.c_void_p),
                ("history_capacity", C.c_int32), ("history_len", C.c_int32), ("info", C.c_int32),
                ("matvecs", C.c_int32), ("launches", C.c_int64)]


class HessenbergStatus(C.Structure):
    _fields_ = [("worst", C.c_uint64), ("first_break", C.c_int32), ("bad", C.c_int32)]


class HessenbergState(C.Structure):
    _fields_ = [("m_max", C.c_int32), ("nshift", C.c_int32), ("done", C.c_int32), ("pad", C.c_int32),
                ("shifts", C.c_void_p), ("beta", C.c_double), ("breakdown_tol", C.c_double),
                ("sinkproj_conj", C.c_void_p), ("rot_c", C.c_void_p), ("rot_s", C.c_void_p), ("vsink", C.c_void_p),
                ("carry", C.c_void_p), ("accum", C.c_void_p), ("green", C.c_void_p), ("residual", C.c_void_p),
                ("status", C.c_void_p)]


class ArnoldiChannel(C.Structure):
    _fields_ = [("sigma", C.c_void_p), ("b", C.c_void_p), ("sink_conj", C.c_void_p), ("V", C.c_void_p),
                ("Hcol", C.c_void_p), ("coeff", C.c_void_p), ("partial", C.c_void_p), ("host", C.c_void_p),
                ("H", C.c_void_p), ("hess", HessenbergState), ("status_host", C.c_void_p), ("work", C.c_void_p),
                ("counters", C.c_void_p), ("V32", C.c_void_p), ("work32", C.c_void_p), ("V32lo", C.c_void_p),
                ("work32lo", C.c_void_p), ("xscatter_offsets", C.c_void_p), ("xscatter_dst", C.c_void_p),
                ("xscatter_sign", C.c_void_p), ("check_dims", C.c_void_p),
                ("check_res", C.c_void_p), ("check_capacity", C.c_int32),
                ("m", C.c_int32), ("breakdown", C.c_int32), ("converged", C.c_int32), ("nchecks", C.c_int32),
                ("pad", C.c_int32), ("beta", C.c_double), ("action_seconds", C.c_double), ("launches", C.c_int64)]


EXPORTS = (
    "c3l_tilde_unpack", "c3l_scatter_padded", "c3l_contract", "c3l_wedge_padded", "c3l_wedge_static_out",
    "c3l_wedge_eom_out", "c3l_wedge_source_out", "c3l_action_prepare", "c3l_static_apply", "c3l_eom_sigma",
    "c3l_eom_sigma_batch",
    "c3l_multi_dot_scratch", "c3l_multi_dot_c", "c3l_multi_dot_r", "c3l_multi_axpy_c", "c3l_multi_axpy_r",
    "c3l_scale_c", "c3l_scale_r", "c3l_precondition", "c3l_hessenberg_shifted", "c3l_hessenberg_coordinates",
    "c3l_hessenberg_coordinates_noalloc", "c3l_gmres", "c3l_gmres_scratch", "c3l_gmres_release", "c3l_gmres_shifted", "c3l_shifted_combine", "c3l_arnoldi", "c3l_hessenberg_advance",
    "c3l_arnoldi_column", "c3l_static_apply_f32", "c3l_eom_sigma_f32", "c3l_action_prepare_f32", "c3l_downcast",
    "c3l_wedge_static_out_f32", "c3l_pair_gemm", "c3l_pair_gemm_df", "c3l_pair_gemm_f32", "c3l_pair_gemm_tc", "c3l_mlp_forward", "c3l_mlp_backward", "c3l_mlp_adam", "c3l_warm_features", "c3l_warm_apply", "c3l_version",
)


def _declare(lib) -> None:
    P, I64, I32, D = C.c_void_p, C.c_int64, C.c_int32, C.c_double
    sig = {
        "c3l_tilde_unpack": [I64, P, P, P, P, P, P, P],
        "c3l_scatter_padded": [I64, P, P, P, P, P, P],
        "c3l_contract": [P, I32, P, P, P],
        "c3l_wedge_padded": [P, I32, P, P],
        "c3l_wedge_static_out": [P, I32, P, P, P, P, P, P, P, P],
        "c3l_wedge_eom_out": [P, I32, P, P, P, P, P],
        "c3l_wedge_static_out_f32": [P, I32, P, P, P, P, P, P, P, P],
        "c3l_wedge_source_out": [P, I32, P, Complex, P, P],
        "c3l_action_prepare": [P, P, P],
        "c3l_static_apply": [P, P, P, P],
        "c3l_eom_sigma": [P, P, P, P],
        "c3l_eom_sigma_batch": [P, I32, P, P, P],
        "c3l_multi_dot_c": [P, I64, I32, P, I64, P, P, P],
        "c3l_multi_dot_r": [P, I64, I32, P, I64, P, P, P],
        "c3l_multi_axpy_c": [P, I64, I32, P, Complex, P, I64, P],
        "c3l_multi_axpy_r": [P, I64, I32, P, D, P, I64, P],
        "c3l_scale_c": [I64, Complex, P, P, P],
        "c3l_scale_r": [I64, D, P, P, P],
        "c3l_precondition": [I64, P, P, P, P, P, P],
        "c3l_hessenberg_shifted": [P, I64, I32, P, I32, D, P, P, P, P],
        "c3l_hessenberg_coordinates": [P, I64, I32, P, I32, D, P, P, P],
        "c3l_hessenberg_coordinates_noalloc": [P, I64, I32, P, I32, D, P, P],
        "c3l_gmres": [P, P],
        "c3l_gmres_shifted": [P, P],
        "c3l_shifted_combine": [I64, Complex, P, P, P, P, P],
        "c3l_static_apply_f32": [P, P, P, P],
        "c3l_eom_sigma_f32": [P, P, P, P],
        "c3l_action_prepare_f32": [P, P, P],
        "c3l_downcast": [I64, P, P, P],
        "c3l_pair_gemm": [P, P, P],
        "c3l_pair_gemm_df": [P, P, P],
        "c3l_pair_gemm_tc": [P, P, P],
        "c3l_pair_gemm_f32": [P, P, P],
        "c3l_mlp_forward": [I64, P, P, P, P],
        "c3l_mlp_backward": [I64, P, P, P, C.c_float, P, P, P, P],
        "c3l_mlp_adam": [P, P, P, P, C.c_float, C.c_float, C.c_float, C.c_float, I32, P, P],
        "c3l_warm_features": [I64, P, P, P, P, P, P, D, D, P, P],
        "c3l_warm_apply": [I64, P, P, P, P, D, P, P],
        "c3l_hessenberg_advance": [P, P, I64, I32, P],
        "c3l_arnoldi_column": [P, I32, P, I64, P, I64, I32, D, P],
        "c3l_arnoldi": [P, I32, I64, P, I32, I32, D, I32, I32, D, P],
    }
    for name, args in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = C.c_int
    lib.c3l_multi_dot_scratch.argtypes = [I32, I64]
    lib.c3l_multi_dot_scratch.restype = I64
    lib.c3l_gmres_scratch.argtypes = [I32, I64]
    lib.c3l_gmres_scratch.restype = I64
    lib.c3l_gmres_release.argtypes = [P]
    lib.c3l_gmres_release.restype = None
    lib.c3l_version.argtypes = []
    lib.c3l_version.restype = C.c_char_p


def load_library(build_if_missing: bool = True):
    """Load (building if needed) the in-tree CUDA library."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = _build.library_path()
    if build_if_missing:
        path = _build.build()
    if not Path(path).exists():
        raise C3LError(f"CUDA library {path} is missing; run c3lindblad_gb300._build.build()")
    lib = C.CDLL(str(path))
    _declare(lib)
    _LIB = lib
    return lib


def lib():
    return load_library()


def check(status: int, what: str) -> None:
    if status != 0:
        raise C3LError(f"{what} failed with c3l_status {status}")


def require_cuda(device=None) -> torch.device:
    if not torch.cuda.is_available():
        raise C3LError("c3lindblad_gb300 needs a CUDA device: there is no CPU fallback")
    dev = torch.device(device if device is not None else "cuda")
    if dev.type != "cuda":
        raise C3LError("c3lindblad_gb300 runs on CUDA devices only")
    return dev


def stream_ptr(device) -> int:
    return torch.cuda.current_stream(device).cuda_stream


def ptr(t: torch.Tensor | None) -> int:
    return 0 if t is None else t.data_ptr()


def cplx(z: complex) -> Complex:
    z = complex(z)
    return Complex(z.real, z.imag)


class Uploader:
    """Keeps device copies of host tables alive and hands out raw pointers.

    Inside ``with uploader.batch():`` tables are placed in a device arena
    (their addresses are known at once) and sent in one copy per arena chunk
    when the block ends; no kernel may read them before the block has ended.
    Outside a batch every table is copied immediately."""

    _CHUNK = 4 << 20
    _ALIGN = 256

    def __init__(self, device):
        self.device = device
        self.keep: list = []
        self._tables: dict = {}  # id(array) -> (array, device copy): one upload per table
        self._pending = None     # [(device byte view, host bytes)] inside a batch
        self._arena = None
        self._used = 0

    @contextlib.contextmanager
    def batch(self):
        if self._pending is not None:  # nested: the outer block sends
            yield self
            return
        self._pending, self._arena, self._used = [], None, 0
        cached = set(self._tables)
        try:
            yield self
            self._send(self._pending)
        except BaseException:
            for key in set(self._tables) - cached:  # never hand out a table that was not sent
                del self._tables[key]
            raise
        finally:
            self._pending, self._arena, self._used = None, None, 0

    def _send(self, pending) -> None:
        groups: dict = {}
        for dst, host in pending:  # by arena chunk (or own allocation)
            base = dst.untyped_storage().data_ptr()
            groups.setdefault(base, []).append((dst, host))
        for items in groups.values():
            if len(items) == 1:
                dst, host = items[0]
                dst.copy_(torch.from_numpy(host.copy()))
                continue
            chunk = items[0][0]
            base = chunk.untyped_storage().data_ptr()
            end = max(d.data_ptr() - base + d.numel() for d, _ in items)
            stage = np.empty(end, dtype=np.uint8)
            for d, h in items:
                off = d.data_ptr() - base
                stage[off:off + h.size] = h
            whole = torch.empty(0, dtype=torch.uint8, device=self.device).set_(chunk.untyped_storage(), 0, (end,))
            whole.copy_(torch.from_numpy(stage))

    def raw(self, arr: np.ndarray) -> torch.Tensor:
        a = np.ascontiguousarray(arr)
        if a.dtype.names is not None or a.dtype == np.int8:
            flat = a.view(np.uint8).reshape(-1)
        elif a.dtype == np.complex128:
            flat = a.view(np.float64).reshape(-1)
        elif a.dtype == np.complex64:
            flat = a.view(np.float32).reshape(-1)
        else:
            flat = a.reshape(-1)
        if self._pending is None:
            t = torch.from_numpy(flat.copy()).to(self.device, non_blocking=False)
        else:
            dtype = torch.from_numpy(flat[:0].copy()).dtype
            nbytes = int(flat.nbytes)
            need = max(self._ALIGN, (nbytes + self._ALIGN - 1) // self._ALIGN * self._ALIGN)
            if need > self._CHUNK // 2:
                dst = torch.empty(need, dtype=torch.uint8, device=self.device)[:nbytes]
            else:
                if self._arena is None or self._used + need > self._CHUNK:
                    self._arena = torch.empty(self._CHUNK, dtype=torch.uint8, device=self.device)
                    self._used = 0
                dst = self._arena[self._used:self._used + nbytes]
                self._used += need
            t = dst.view(dtype).view(flat.shape)
            if nbytes:
                self._pending.append((dst, flat.view(np.uint8).reshape(-1)))
        self.keep.append(t)
        return t

    def table(self, arr) -> torch.Tensor:
        """Device copy of a (read-only) program table, uploaded once per array."""
        hit = self._tables.get(id(arr))
        if hit is not None and hit[0] is arr:
            return hit[1]
        t = self.raw(arr)
        self._tables[id(arr)] = (arr, t)
        return t

    def ptr(self, arr) -> int:
        """Device address of a (read-only) program table, uploaded once: actions
        built from the same tables share them, which batched launches require."""
        if arr is None:
            return 0
        if len(arr) == 0:
            return 0
        return self.table(arr).data_ptr()


def wedge_stage(up: Uploader, stage) -> WedgeStage:
    st = WedgeStage()
    if stage is None:
        st.ntiles = 0
        return st
    st.blocks = up.ptr(stage.blocks)
    st.instances = up.ptr(stage.instances)
    st.tiles = up.ptr(stage.tiles)
    st.ntiles = len(stage.tiles)
    st.elements = up.ptr(stage.elements) if stage.elements is not None else 0
    st.digits = up.ptr(stage.digits) if stage.digits is not None else 0
    st.width = int(stage.width)
    return st


def pair_program(up: Uploader, program, name: str | None, kernel: int = PAIR_SIMT, status: int = 0) -> PairProgram:
    """The pair GEMMs feeding stage ``<name>_pairs`` (none when ``name`` is None);
    ``kernel`` PAIR_TCGEN05 runs an FP32 workspace's GEMMs on the tensor cores."""
    pp = PairProgram()
    pairs = program.pairs.get(name) if name else None
    if pairs is None or pairs.tiles.size == 0:
        pp.ntiles = 0
        return pp
    pp.groups = up.ptr(pairs.groups)
    pp.aoff = up.ptr(pairs.aoff)
    pp.roff = up.ptr(pairs.roff)
    pp.tiles = up.ptr(pairs.tiles)
    pp.ntiles = pairs.tiles.size
    pp.base = program.ws_size
    if pairs.tiles_tc is not None and pairs.tiles_tc.size:
        pp.tiles_tc = up.ptr(pairs.tiles_tc)
        pp.ntiles_tc = pairs.tiles_tc.size
    pp.kernel = int(kernel)
    pp.status = int(status)
    return pp


def build_action(up: Uploader, program, vectors_ptr: int, ws: torch.Tensor, levels_cls: str | None,
                 padded_names: list, out_name: str | None, scatter, pairs: str | None = None,
                 pair_kernel: int = PAIR_SIMT, pair_status: int = 0) -> Action:
    """``pairs``: run the pair GEMMs of that stage before the output stage
    (``ws`` then holds the workspace followed by the pair buffer)."""
    if pairs is not None and ws.numel() < program.ws_size + program.pair_size:
        raise C3LError("the workspace has no room for the pair buffer")
    a = Action()
    a.n = program.n
    levels = program.levels.get(levels_cls, []) if levels_cls else []
    if len(levels) > 8:
        raise C3LError("too many contraction levels")
    a.nlevels = len(levels)
    for i, lv in enumerate(levels):
        a.levels[i].tasks = up.ptr(lv.tasks)
        a.levels[i].tiles = up.ptr(lv.tiles)
        a.levels[i].ntiles = len(lv.tiles)
    stages = [program.stages[nm] for nm in padded_names if nm in program.stages]
    if len(stages) > 1:  # independent padded stages share one launch
        from .compiler import merge_padded

        key = tuple(st.name for st in stages)
        cache = program.__dict__.setdefault("_merged_padded", {})
        if key not in cache:
            cache[key] = merge_padded(stages, program.n)
        stages = [cache[key]]
    if len(stages) > 4:
        raise C3LError("too many padded stages")
    a.npadded = len(stages)
    for i, s in enumerate(stages):
        a.padded[i] = wedge_stage(up, s)
    a.out = wedge_stage(up, program.stages.get(out_name) if out_name else None)
    a.pairs = pair_program(up, program, pairs, pair_kernel, pair_status)
    a.vectors = vectors_ptr
    a.ws = ws.data_ptr()
    if scatter is not None:
        a.scatter_count = scatter.dst.size
        a.scatter_dst = up.ptr(scatter.dst)
        a.scatter_pos = up.ptr(scatter.pos)
        a.scatter_sign = up.ptr(scatter.sign)
    else:
        a.scatter_count = 0
    return a


class LaunchCounter:
    """Counts this library's kernel launches issued through the host wrappers."""

    count = 0

    @classmethod
    def add(cls, k: int) -> None:
        cls.count += k

    @classmethod
    def reset(cls) -> int:
        c = cls.count
        cls.count = 0
        return c


CLUSTER_LEVEL_MAX_TILES = 16  # levels this small at the end of the list run as one cluster launch
                              # (16-CTA clusters on GB300; the count is an estimate where only 8 are allowed)


SPLIT_SCATTER = 1 << 20  # scatter entries from which c3l_static_apply unpacks and scatters in two launches


def static_launches(a: Action) -> int:
    """Kernels of one c3l_static_apply: the unpack and the scatter (fused
    below SPLIT_SCATTER entries) replace the action's scatter."""
    if a.scatter_count >= SPLIT_SCATTER:
        return action_launches(a) + 1
    return action_launches(a) + (0 if a.scatter_count > 0 else 1)


def action_launches(a: Action) -> int:
    k = 1 if a.scatter_count > 0 else 0
    tail = a.nlevels
    while tail > 0 and a.levels[tail - 1].ntiles <= CLUSTER_LEVEL_MAX_TILES:
        tail -= 1
    if a.nlevels - tail < 2:
        tail = a.nlevels
    k += sum(1 for i in range(tail) if a.levels[i].ntiles > 0) + (1 if tail < a.nlevels else 0)
    k += sum(1 for i in range(a.npadded) if a.padded[i].ntiles > 0)
    k += 1 if a.pairs.ntiles > 0 else 0
    k += 1 if a.out.ntiles > 0 else 0
    return k
