"""CPU oracle of the warm-start MLP (test infrastructure only).

Float64 restatement of ``c3lindblad_gb300/csrc/c3l_mlp.cu`` with the same
BF16 roundings (inputs, weights and the two hidden activations are rounded
to BF16 before use), so the device forward pass and its gradients can be
checked elementwise.  The reference has no counterpart: its Newton solve
starts from zero amplitudes (``src/c3l/cc/component_solver.py:121-122``).
"""

from __future__ import annotations

import numpy as np

F, H, O = 16, 32, 2
OFFSETS = {}
_o = 0
for _name, _size in (("W1", H * F), ("b1", H), ("W2", H * H), ("b2", H), ("W3", O * H), ("b3", O)):
    OFFSETS[_name] = (_o, _size)
    _o += _size
PARAMS = _o


def bf16_round(x: np.ndarray) -> np.ndarray:
    """Round float32 values to the nearest BF16 (ties to even), returned as float64."""
    a = np.asarray(x, dtype=np.float32).copy()
    bits = a.view(np.uint32)
    lsb = (bits >> 16) & 1
    bits = (bits + 0x7FFF + lsb) & 0xFFFF0000
    return bits.view(np.float32).astype(np.float64)


def unpack(params: np.ndarray) -> dict:
    p = np.asarray(params, dtype=np.float64)
    out = {}
    for name, (off, size) in OFFSETS.items():
        out[name] = p[off:off + size]
    out["W1"] = out["W1"].reshape(H, F)
    out["W2"] = out["W2"].reshape(H, H)
    out["W3"] = out["W3"].reshape(O, H)
    return out


def forward(params_bf16: np.ndarray, X_bf16: np.ndarray):
    w = unpack(params_bf16)
    a1 = X_bf16 @ w["W1"].T + w["b1"]
    h1 = bf16_round(np.tanh(a1))
    a2 = h1 @ w["W2"].T + w["b2"]
    h2 = bf16_round(np.tanh(a2))
    y = h2 @ w["W3"].T + w["b3"]
    return y, (h1, h2)


def loss_and_grad(params_bf16: np.ndarray, X_bf16: np.ndarray, T: np.ndarray, W: np.ndarray | None = None):
    """Weighted squared error sum_s w_s |y_s - t_s|^2 / sum w and its gradient."""
    w = unpack(params_bf16)
    n = X_bf16.shape[0]
    ws = np.ones(n) if W is None else np.asarray(W, dtype=np.float64)
    y, (h1, h2) = forward(params_bf16, X_bf16)
    e = y - T
    loss = float(np.sum(ws[:, None] * e * e))
    dy = 2.0 * ws[:, None] * e / ws.sum()
    g = {"W3": dy.T @ h2, "b3": dy.sum(0)}
    d2 = (dy @ w["W3"]) * (1.0 - h2 * h2)
    g["W2"] = d2.T @ h1
    g["b2"] = d2.sum(0)
    d1 = (d2 @ w["W2"]) * (1.0 - h1 * h1)
    g["W1"] = d1.T @ X_bf16
    g["b1"] = d1.sum(0)
    flat = np.concatenate([g[name].reshape(-1) for name in OFFSETS])
    return loss, flat
