"""The CUDA library builds for sm_103a, loads, and exports the declared C ABI."""

from __future__ import annotations

import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def declared_symbols():
    text = (ROOT / "include" / "c3l_gb300.h").read_text()
    return sorted(set(re.findall(r"^\s*(?:c3l_status|int64_t|const char\*)\s+(c3l_\w+)\s*\(", text, re.M)))


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
