"""Shared test setup: markers, native build, golden fixtures."""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
GOLDEN = Path(__file__).resolve().parent / "golden"
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(Path(__file__).resolve().parent))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a)")
    # The product library and the CPU oracle are built before collection so
    # that every test runs against freshly compiled native code.
    import __graft_entry__ as G

    G._load_build_module().build()
    from oracle import oracle as O

    O.build_port()


def golden_names():
    return sorted(p.stem for p in GOLDEN.glob("*.npz"))


def load_golden(name: str) -> dict[str, np.ndarray]:
    with np.load(GOLDEN / f"{name}.npz") as z:
        return {k: z[k] for k in z.files}


def rel_err(x: np.ndarray, ref: np.ndarray, floor: float = 1e-6) -> float:
    """Componentwise relative error with a floor of `floor` x max|ref|.

    The floor keeps cancellation-sized entries (fill that ends near zero) from
    dominating; every other entry is compared relative to itself."""
    x = np.asarray(x, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    scale = np.maximum(np.abs(ref), floor * max(np.abs(ref).max(), 1e-300))
    return float(np.max(np.abs(x - ref) / scale)) if ref.size else 0.0


def norm_err(x: np.ndarray, ref: np.ndarray) -> float:
    """Normwise relative error max|x - ref| / max|ref| (solution vectors)."""
    x = np.asarray(x, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    return float(np.max(np.abs(x - ref)) / max(np.abs(ref).max(), 1e-300)) if ref.size else 0.0


def has_gpu() -> bool:
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:  # pragma: no cover
        return False


@pytest.fixture(scope="session")
def cuda():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda:0")
