"""The CUDA library builds for sm_103a, loads, and exports the declared C ABI."""

from __future__ import annotations

import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]


def declared_symbols():
    text = (ROOT / "include" / "c3l_gb300.h").read_text()
    return sorted(set(re.findall(r"^\s*(?:c3l_status|int64_t|void|const char\*)\s+(c3l_\w+)\s*\(", text, re.M)))


def test_header_declares_entry_points():
    names = declared_symbols()
    assert "c3l_static_apply" in names and "c3l_eom_sigma" in names and "c3l_hessenberg_shifted" in names
    assert len(names) >= 20


def test_library_loads_and_exports_every_declared_symbol():
    from c3lindblad_gb300 import runtime

    lib = runtime.load_library()
    for name in declared_symbols():
        assert hasattr(lib, name), name
    assert set(runtime.EXPORTS) == set(declared_symbols())
    assert b"sm_103a" in lib.c3l_version()


def test_device_entry_points_refuse_without_cuda():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("GPU present")
    from c3lindblad_gb300 import runtime

    with pytest.raises(runtime.C3LError):
        runtime.require_cuda()


def test_bad_arguments_are_rejected_before_launch():
    """Null pointers and bad sizes return C3L_ERR_ARGUMENT without touching a GPU."""
    from c3lindblad_gb300 import runtime

    lib = runtime.load_library()
    assert lib.c3l_scatter_padded(5, None, None, None, None, None, None) == 1
    assert lib.c3l_multi_dot_r(None, 0, 1, None, 10, None, None, None) == 1
    assert lib.c3l_hessenberg_shifted(None, 4, 4, None, 1, 1.0, None, None, None, None) == 1
    assert lib.c3l_static_apply(None, None, None, None) == 1
    assert lib.c3l_eom_sigma(None, None, None, None) == 1


def test_krylov_drivers_reject_bad_arguments_before_launch():
    """The drivers and the incremental shifted solves validate their structs on the host."""
    import ctypes as C

    from c3lindblad_gb300 import runtime

    lib = runtime.load_library()
    assert lib.c3l_gmres(None, None) == 1
    assert lib.c3l_gmres_shifted(None, None) == 1
    assert lib.c3l_gmres_shifted(C.byref(runtime.GmresShiftedArgs()), None) == 1  # all pointers null
    assert lib.c3l_arnoldi(None, 0, 10, None, 1, 4, 1e-10, 1, 8, 1e-14, None) == 1
    assert lib.c3l_hessenberg_advance(None, None, 5, 4, None) == 1
    st = runtime.HessenbergState()  # zero sizes and null buffers
    assert lib.c3l_hessenberg_advance(C.byref(st), None, 5, 4, None) == 1
    assert lib.c3l_shifted_combine(-1, runtime.cplx(1.0), None, None, None, None, None) == 1
    assert lib.c3l_shifted_combine(0, runtime.cplx(1.0), None, None, None, None, None) == 0  # empty is a no-op
    # capacity limits are stated in the header and enforced
    assert lib.c3l_arnoldi(None, 1, 10, None, 1, 5000, 1e-10, 1, 8, 1e-14, None) == 1
    assert lib.c3l_gmres_scratch(0, 10) == 0
    assert lib.c3l_gmres_scratch(40, 20933) >= 42


def test_gmres_graph_release_accepts_null():
    from c3lindblad_gb300 import runtime

    lib = runtime.load_library()
    lib.c3l_gmres_release(None)  # no-op


def test_uploader_batch_places_every_table_byte_for_byte():
    """Tables uploaded inside ``Uploader.batch()`` share arena chunks and are sent
    in one copy per chunk when the block ends: every table must arrive intact
    (dtype, shape, bytes), whatever its type, size or alignment (run on the CPU
    device: the same placement and copy logic as on the GPU)."""
    import torch
    from c3lindblad_gb300 import runtime as rt

    rng = np.random.default_rng(11)
    rec = np.zeros(7, dtype=[("a", "<i8"), ("b", "<f8"), ("c", "i1")])
    rec["a"] = np.arange(7)
    rec["b"] = rng.normal(size=7)
    arrays = [
        rng.integers(-5, 5, size=1000).astype(np.int64),
        rng.normal(size=333),
        (rng.normal(size=17) + 1j * rng.normal(size=17)).astype(np.complex128),
        (rng.normal(size=9) + 1j * rng.normal(size=9)).astype(np.complex64),
        rng.integers(-3, 3, size=13).astype(np.int8),
        rec,
        np.zeros(0, np.int32),
        rng.integers(0, 2, size=5).astype(bool),
        rng.normal(size=(3, 5)),                               # 2-D
        rng.integers(0, 9, size=(rt.Uploader._CHUNK // 8)),    # larger than half a chunk: own allocation
        rng.normal(size=rt.Uploader._CHUNK // 16),              # fills half a chunk: opens a second chunk
        np.arange(3, dtype=np.uint16),
    ]
    up = rt.Uploader(torch.device("cpu"))
    with up.batch():
        outs = [up.raw(a) for a in arrays]
        cached = up.table(arrays[1])
    assert up.table(arrays[1]) is cached
    for a, t in zip(arrays, outs):
        host = np.ascontiguousarray(a)
        assert t.numel() * t.element_size() == host.nbytes
        assert t.cpu().numpy().tobytes() == host.tobytes()
    # a failed block leaves no cached table behind
    fresh = np.arange(5.0)
    try:
        with up.batch():
            up.table(fresh)
            raise RuntimeError("stop")
    except RuntimeError:
        pass
    assert id(fresh) not in up._tables
    # outside a batch: immediate copies
    t = up.raw(arrays[0])
    assert t.numpy().tobytes() == arrays[0].tobytes()
