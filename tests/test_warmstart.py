"""Learned warm start: gradients against the CPU oracle, and its gain on held-out models."""

from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

from oracle import mlp_oracle as mo

FAMILY = Path(__file__).resolve().parent / "golden" / "warmstart_siam.npz"


def _random_problem(n=64, seed=0):
    rng = np.random.default_rng(seed)
    params = (0.4 * rng.normal(size=mo.PARAMS)).astype(np.float32)
    X = rng.normal(size=(n, mo.F)).astype(np.float32)
    T = rng.normal(size=(n, mo.O)).astype(np.float32)
    return params, X, T


def test_oracle_gradient_matches_finite_differences():
    params, X, T = _random_problem()
    # smooth check without BF16 rounding: differentiate the float64 network
    p = params.astype(np.float64)
    Xd = X.astype(np.float64)

    def loss(q):
        w = mo.unpack(q)
        h1 = np.tanh(Xd @ w["W1"].T + w["b1"])
        h2 = np.tanh(h1 @ w["W2"].T + w["b2"])
        y = h2 @ w["W3"].T + w["b3"]
        return np.sum((y - T) ** 2) / X.shape[0]

    saved = mo.bf16_round
    mo.bf16_round = lambda a: np.asarray(a, dtype=np.float64)
    try:
        _, g = mo.loss_and_grad(p, Xd, T)
    finally:
        mo.bf16_round = saved
    rng = np.random.default_rng(1)
    for k in rng.choice(mo.PARAMS, size=25, replace=False):
        e = np.zeros_like(p)
        e[k] = 1e-6
        fd = (loss(p + e) - loss(p - e)) / 2e-6
        assert abs(fd - g[k]) <= 1e-6 * max(1.0, abs(fd))


def test_bf16_rounding_is_round_to_nearest_even():
    x = np.array([1.0, 1.00390625, 1.01171875, -3.14159], np.float32)
    r = mo.bf16_round(x)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.015625
    assert abs(r[3] + 3.140625) < 1e-12


@pytest.mark.gpu
def test_device_forward_and_gradient_match_oracle(cuda_device):
    torch = pytest.importorskip("torch")
    from c3lindblad_gb300.warmstart import MLPDevice

    params, X, T = _random_problem(n=300, seed=3)
    mlp = MLPDevice(params, cuda_device)
    Xb = torch.from_numpy(X).to(cuda_device).to(torch.bfloat16)
    Td = torch.from_numpy(T).to(cuda_device)
    pb = mo.bf16_round(params)
    xb = Xb.float().cpu().numpy().astype(np.float64)
    y_dev = mlp.forward(Xb).cpu().numpy()
    y_ref, _ = mo.forward(pb, xb)
    assert np.max(np.abs(y_dev - y_ref)) <= 1e-4 * max(1.0, np.max(np.abs(y_ref)))
    g_dev, loss_dev = mlp.gradient(Xb, Td)
    loss_ref, g_ref = mo.loss_and_grad(pb, xb, T.astype(np.float64))
    g_dev = g_dev.cpu().numpy()
    assert abs(loss_dev.item() - loss_ref) <= 1e-4 * loss_ref
    assert np.max(np.abs(g_dev - g_ref)) <= 1e-4 * np.max(np.abs(g_ref))


@pytest.mark.gpu
def test_learned_warm_start_lowers_the_starting_residual_on_held_out_models(cuda_device):
    """Train on 16 seeded models, evaluate on 8 others.

    What the network gains: a starting point whose FP64 residual is below the
    zero guess and below the first-order (Jacobi) guess, both safeguarded by
    the same backtracking.  The converged answer never depends on it: both
    solves reach the same root to 1e-8.
    """
    if not FAMILY.exists():
        pytest.skip("model family file missing")
    torch = pytest.importorskip("torch")
    from c3lindblad_gb300 import solve_component_ccsd
    from c3lindblad_gb300.krylov import DeviceVectors
    from c3lindblad_gb300.warmstart import PARAMS, LearnedWarmStart, collect, load_family, train

    problems = load_family(FAMILY, cuda_device)
    X, T = collect(problems[:16])
    ws, hist = train(X, T, epochs=300, lr=3e-3)
    assert hist[-1] < 0.75 * hist[0]
    first = LearnedWarmStart(np.zeros(PARAMS, np.float32))
    vec = DeviceVectors(cuda_device)
    ratios_first, ratios_learned = [], []
    for p in problems[-8:]:
        a = solve_component_ccsd(p, precision="mixed")
        if not a.converged:
            continue  # strongly coupled draws the zero-guess Newton solve does not converge on
        ops = p.ops
        r = torch.empty(ops.D, dtype=torch.float64, device=cuda_device)
        ops.residual(torch.zeros(ops.D, dtype=torch.float64, device=cuda_device), r)
        r0 = vec.norm_r(r)
        ops.residual(first.initial_variables(p), r)
        r1 = vec.norm_r(r)
        ops.residual(ws.initial_variables(p), r)
        rl = vec.norm_r(r)
        ratios_first.append(r1 / r0)
        ratios_learned.append(rl / r0)
        b = solve_component_ccsd(p, precision="mixed", warm_start=ws)
        assert b.converged and b.packed_residual_norm <= 1e-10
        # two Newton solves stopped by the same residual test agree to about
        # cond(J) times the tolerance, not to rounding
        assert np.max(np.abs(a.amplitudes - b.amplitudes)) <= 5e-8 * np.max(np.abs(a.amplitudes))
    assert len(ratios_learned) >= 4
    print(f"held-out starting residual / zero-guess residual: first-order {np.mean(ratios_first):.3f}, "
          f"learned {np.mean(ratios_learned):.3f}")
    assert max(ratios_learned) <= 1.0
    assert np.mean(ratios_learned) < 1.0
    assert np.mean(ratios_learned) <= np.mean(ratios_first)
