"""The pair-GEMM kernels (``c3l_pair_gemm`` / ``_df`` / ``_f32`` / ``_tc``) against NumPy.

Each group multiplies K gathered operand rows: P[i, j] = sum_k A_k[i] R_k[j]
with A_k = ws[aoff[k] : aoff[k] + M] and R_k = ws[roff[k] : roff[k] + N].  The
shapes cover ragged tiles (M, N not multiples of 64), single rows and columns,
chunks of fewer than 8 anchors, and rows shared between groups.
"""

from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from c3lindblad_gb300 import compiler

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

# (M, N, K); the CUDA-core tiles come from compiler.pair_tiles, so these cover
# every shape: 64 x 64 (65 x 65), 32 x 128 (27 x 729), 128 x 32 (729 x 27),
# 16 x 256 (1 x 300, 11 x 200), 256 x 16 (4225 x 65), and the one-column
# tiles without (300 x 1, 2000 x 1) and with anchor splitting (700 x 1 x 37)
SHAPES = [(1, 1, 1), (3, 7, 2), (64, 64, 8), (65, 65, 9), (130, 17, 23), (1, 300, 5), (300, 1, 5),
          (197, 201, 37), (4225, 65, 3), (27, 729, 9), (729, 27, 12), (11, 200, 17), (2000, 1, 6),
          (700, 1, 37), (33, 1, 16)]


def _program(rng, ws_size: int):
    groups = np.zeros(len(SHAPES), compiler.PAIR_GROUP_DTYPE)
    aoff, roff, tiles, tiles_tc = [], [], [], []
    p = 0
    for g, (M, N, K) in enumerate(SHAPES):
        groups[g] = (p, len(aoff), len(aoff) + K, M, N)
        aoff.extend(int(v) for v in rng.integers(0, ws_size - M + 1, K))
        roff.extend(int(v) for v in rng.integers(0, ws_size - N + 1, K))
        tiles.extend((g, m0, n0, shape) for m0, n0, shape in compiler.pair_tiles(M, N, K))
        for m0 in range(0, M, compiler.PAIR_TILE_TC[0]):
            for n0 in range(0, N, compiler.PAIR_TILE_TC[1]):
                tiles_tc.append((g, m0, n0, 0))
        p += M * N

    def table(rows):
        t = np.zeros(len(rows), compiler.PAIR_TILE_DTYPE)
        for i, row in enumerate(rows):
            t[i] = row
        return t

    return groups, np.asarray(aoff, np.int64), np.asarray(roff, np.int64), table(tiles), table(tiles_tc), p


def _expected(ws, groups, aoff, roff):
    out = []
    for g in groups:
        k = np.arange(int(g["kbegin"]), int(g["kend"]))
        A = ws[aoff[k][:, None] + np.arange(int(g["M"]))[None, :]]
        R = ws[roff[k][:, None] + np.arange(int(g["N"]))[None, :]]
        out.append((A.T @ R).reshape(-1))
    return np.concatenate(out)


@pytest.mark.parametrize("dtype", ["f64", "df", "f32", "tc"])
def test_pair_gemm_matches_numpy(dtype, cuda_device):
    from c3lindblad_gb300 import runtime as rt

    lib = rt.lib()
    rng = np.random.default_rng(7)
    ws_size = 20000
    groups, aoff, roff, tiles, tiles_tc, psize = _program(rng, ws_size)
    ws = rng.normal(size=ws_size) + 1j * rng.normal(size=ws_size)
    want = _expected(ws, groups, aoff, roff)
    cdt = torch.complex64 if dtype in ("f32", "tc") else torch.complex128
    buf = torch.full((ws_size + psize,), complex("nan"), dtype=cdt, device=cuda_device)
    buf[:ws_size] = torch.from_numpy(ws).to(cuda_device, cdt)
    keep = [torch.from_numpy(a.view(np.uint8).copy()).to(cuda_device) for a in (groups, aoff, roff, tiles, tiles_tc)]
    status = torch.zeros(1, dtype=torch.int32, device=cuda_device)
    pp = rt.PairProgram()
    pp.groups, pp.aoff, pp.roff, pp.tiles, pp.tiles_tc = (k.data_ptr() for k in keep)
    pp.ntiles = tiles.size
    pp.ntiles_tc = tiles_tc.size
    pp.base = ws_size
    pp.status = status.data_ptr()
    fn = {"f64": lib.c3l_pair_gemm, "df": lib.c3l_pair_gemm_df, "f32": lib.c3l_pair_gemm_f32,
          "tc": lib.c3l_pair_gemm_tc}[dtype]
    assert fn(C.byref(pp), buf.data_ptr(), torch.cuda.current_stream(cuda_device).cuda_stream) == 0
    torch.cuda.synchronize(cuda_device)
    got = buf[ws_size:].cpu().numpy().astype(np.complex128)
    assert np.all(np.isfinite(got))  # every P entry written
    # per-entry bound: |error| <= c eps sum_k |A_k[i]| |R_k[j]|
    assert int(status.item()) == 0
    # FP64: reassociation only; double-float: products to 2^-46 and TwoSum sums;
    # FP32 and split-TF32 (three TF32 MMAs per real product): about 2^-21 per product
    tol = {"f64": 1e-13, "df": 1e-12, "f32": 3e-6, "tc": 3e-6}[dtype]
    scale = _expected(np.abs(ws), groups, aoff, roff).real
    assert np.all(np.abs(got - want) <= tol * scale)
    # the workspace itself is untouched
    assert np.array_equal(buf[:ws_size].cpu().numpy().astype(np.complex128),
                          ws if dtype not in ("f32", "tc") else ws.astype(np.complex64).astype(np.complex128))
