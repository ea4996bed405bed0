"""Allocation-free reduced-coordinate solve, checked against the allocating entry point.

``c3l_hessenberg_coordinates_noalloc`` serves callers that cannot allocate
device memory themselves -- for example a host application that owns the
whole device-memory budget and hands the library only input and output
buffers.  It keeps its scratch in a fixed array inside the library, so this
test calls it twice in a row, on two different problems, and compares each
result with ``c3l_hessenberg_coordinates`` given caller-allocated scratch.
This file is collected last so a failure here never hides another test.
"""

from __future__ import annotations

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _problem(rng, m: int, nshift: int, scale: float = 1.0, damping: float = 0.0):
    """A Hessenberg matrix with positive subdiagonal; ``damping`` moves its
    diagonal to Im = -damping, as for a dissipative operator, which keeps
    z I - H well conditioned for the shifts (Im z = 0.05) at large m."""
    H = scale * np.triu(rng.normal(size=(m + 1, m)) + 1j * rng.normal(size=(m + 1, m)), -1)
    H[np.arange(1, m + 1), np.arange(m)] = np.abs(H[np.arange(1, m + 1), np.arange(m)]) + 0.5 * scale
    H[np.arange(m), np.arange(m)] -= 1j * damping
    shifts = np.linspace(-4.0, 4.0, nshift) + 0.05j
    return H, shifts


def test_noalloc_coordinates_match_allocating_entry_point(cuda_device):
    from c3lindblad_gb300 import runtime

    lib = runtime.load_library()
    stream = torch.cuda.current_stream(cuda_device).cuda_stream
    rng = np.random.default_rng(2024)
    # calls in a row; each problem is larger than the one before, so stale
    # scratch from an earlier call would show up in its result.  The last one
    # needs 60 * 400 * 401 / 2 entries, more than the fixed scratch holds, so
    # its shifts run in three chunks (26, 26, 8) that reuse the array in order.
    for m, nshift, beta, scale, damping in ((40, 29, 1.7, 1.0, 0.0), (96, 53, 0.6, 1.0, 0.0),
                                            (400, 60, 1.1, 0.1, 1.0)):
        H, shifts = _problem(rng, m, nshift, scale, damping)
        Hd = torch.from_numpy(np.ascontiguousarray(H)).to(cuda_device)
        zd = torch.from_numpy(shifts).to(cuda_device)
        scratch = torch.empty(nshift * m * (m + 1) // 2, dtype=torch.complex128, device=cuda_device)
        want = torch.empty((nshift, m), dtype=torch.complex128, device=cuda_device)
        st = lib.c3l_hessenberg_coordinates(Hd.data_ptr(), m, m, zd.data_ptr(), nshift, beta, scratch.data_ptr(),
                                            want.data_ptr(), stream)
        assert st == 0
        got = torch.full((nshift, m), complex("nan"), dtype=torch.complex128, device=cuda_device)
        st = lib.c3l_hessenberg_coordinates_noalloc(Hd.data_ptr(), m, m, zd.data_ptr(), nshift, beta, got.data_ptr(),
                                                    stream)
        assert st == 0
        torch.cuda.synchronize(cuda_device)
        w = want.cpu().numpy()
        g = got.cpu().numpy()
        assert np.all(np.isfinite(g))
        assert np.max(np.abs(g - w)) <= 1e-12 * np.max(np.abs(w))
        # and both solve (z I - H_m) y = beta e1
        e1 = np.zeros(m, complex)
        e1[0] = beta
        for s in (0, nshift // 2, nshift - 1):
            y = np.linalg.solve(shifts[s] * np.eye(m) - H[:m, :m], e1)
            assert np.max(np.abs(g[s] - y)) <= 1e-9 * np.max(np.abs(y))


def test_noalloc_rejects_sizes_beyond_its_scratch(cuda_device):
    from c3lindblad_gb300 import runtime

    lib = runtime.load_library()
    m = 3000  # m (m + 1) / 2 exceeds the fixed scratch; rejected before any launch
    H = torch.zeros(4, dtype=torch.complex128, device=cuda_device)
    out = torch.zeros(4, dtype=torch.complex128, device=cuda_device)
    st = lib.c3l_hessenberg_coordinates_noalloc(H.data_ptr(), m, m, H.data_ptr(), 1, 1.0, out.data_ptr(),
                                                torch.cuda.current_stream(cuda_device).cuda_stream)
    assert st == 3  # C3L_ERR_CAPACITY
