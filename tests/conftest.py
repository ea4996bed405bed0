"""Shared fixtures: golden files and the GPU marker."""

from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
GOLDEN = ROOT / "tests" / "golden"
for p in (str(ROOT), str(ROOT / "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300) and the built CUDA library")


def golden_names(with_solution: bool = False, with_eom: bool = False, with_green: bool = False,
                 compact: bool = False):
    """Fixtures with full golden vectors (default) or compact sampled ones."""
    names = []
    for f in sorted(GOLDEN.glob("*.golden.npz")):
        name = f.name[: -len(".golden.npz")]
        files = np.load(f).files
        if ("compact" in files) != compact:
            continue
        if with_solution and "solution_amplitudes" not in files:
            continue
        if with_eom and "eomp_sigma" not in files and "eomp_sigma_sample" not in files:
            continue
        if with_green and "green_retarded" not in files:
            continue
        names.append(name)
    return names


def eom_amplitudes(g):
    """Amplitudes at which the reference evaluated its EOM goldens."""
    return g["eom_amplitudes"] if "eom_amplitudes" in g else g["solution_amplitudes"]


def load(name: str):
    from c3lindblad_gb300.spec import ProblemSpec

    spec = ProblemSpec.load(GOLDEN / f"{name}.spec.npz")
    gold = dict(np.load(GOLDEN / f"{name}.golden.npz"))
    return spec, gold


def relerr(a, b) -> float:
    a = np.asarray(a)
    b = np.asarray(b)
    scale = max(float(np.max(np.abs(b))), 1e-300)
    return float(np.max(np.abs(a - b))) / scale


@pytest.fixture(scope="session")
def cuda_device():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda:0")
