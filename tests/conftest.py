import json
import sys
from pathlib import Path

import numpy as np
import pytest

REPO = Path(__file__).resolve().parents[1]
for p in (REPO, REPO / "tests", REPO / "intel-qs_gb300"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))

GOLDEN = REPO / "tests" / "golden" / "golden.npz"

# Parity bars (per-amplitude max abs error against the reference's CPU path).
TOL_DP = 1e-12
TOL_SP = 2e-5


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the libiqsg kernels)")


@pytest.fixture(scope="session")
def golden():
    z = np.load(GOLDEN, allow_pickle=False)
    return {k: z[k] for k in z.files}


def golden_cases(store, prefix=""):
    names = sorted({k.split("/")[0] for k in store})
    return [n for n in names if n.startswith(prefix) and f"{n}/ops" in store]


def case_meta(store, name):
    return json.loads(str(store[f"{name}/meta"]))


def case_ops(store, name):
    return json.loads(str(store[f"{name}/ops"]))


def compare_final(store, name, state, tol):
    """Max abs difference between a full final state and the golden one (sampled cases:
    compares the stored indices and the norm / fourth-moment checksums)."""
    ref = store[f"{name}/final"]
    if f"{name}/final_idx" in store:
        idx = store[f"{name}/final_idx"]
        err = float(np.max(np.abs(state[idx] - ref)))
        n2 = float(np.vdot(state, state).real)
        s4 = float(np.sum(np.abs(state.astype(np.complex128)) ** 4))
        err = max(err, abs(n2 - float(store[f"{name}/final_norm2"])),
                  abs(s4 - float(store[f"{name}/final_sum4"])))
        return err
    return float(np.max(np.abs(state - ref)))


def gpu_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False
