"""Autotuner for fused passes: picks the sweep width (target qubits per pass), the pass
kernel (direct loads or the bulk-copy pipeline) and, for emulated ComplexDP, the share of
warps that use the FP64 pipe, by timing a representative layer on the register itself.
The choice changes the time, and the results at most by rounding.

    best = tune_fusion(reg)          # reg: a QubitRegister holding a dense state
    reg.SetSweepWidth(best["width"]); reg.SetSweepPipeline(best["pipeline"])
    reg.SetNativeShare(best["native_share"])

Choices are cached per (qubits, precision, math, device) for the process.
"""
from __future__ import annotations

import time
from typing import Dict, Iterable, Optional, Tuple

import numpy as np

from .qureg import QubitRegister

_CACHE: Dict[Tuple, dict] = {}


def _layer(reg: QubitRegister, rng: np.random.Generator) -> None:
    n = reg.NumQubits()
    for q in range(n):
        z = rng.standard_normal((2, 2)) + 1j * rng.standard_normal((2, 2))
        u, _ = np.linalg.qr(z)
        reg.Apply1QubitGate(q, u)
    for q in range(0, n - 1, 2):
        reg.ApplyCPauliZ(q, q + 1)
    for q in range(1, n - 1, 2):
        reg.ApplyCPauliZ(q, q + 1)


def _device_key() -> str:
    try:
        import torch
        return torch.cuda.get_device_name()
    except Exception:
        return "cuda"


def tune_fusion(reg: QubitRegister, widths: Iterable[int] = (1, 2, 3, 4), pipelines: Iterable[bool] = (False, True),
                shares: Iterable[int] = (), trials: int = 2, apply: bool = True, seed: int = 99) -> dict:
    """Time one layer (Haar U on every qubit + CZ bricks) for every (width, pipeline) -- and
    for emulated ComplexDP every native share in `shares` with direct loads (none by
    default: on GB300 every share above 0 measured slower) -- and return
    the fastest, as {"width", "pipeline", "native_share", "ms", "table"}. With apply=True the
    register keeps the chosen settings. The register's state is changed by the trial layers."""
    key = (reg.NumQubits(), reg.precision, reg._math, _device_key())
    emulated = reg.precision == "DP" and reg._math == 1
    if key in _CACHE:
        best = _CACHE[key]
    else:
        rng = np.random.default_rng(seed)
        was = reg.IsFusionEnabled()
        reg.TurnOnFusion()
        cands = []
        for w in widths:
            if emulated and w > 3:
                continue  # emulated passes hold at most 3 target qubits
            for pl in pipelines:
                if pl and reg.NumQubits() < 16:
                    continue
                cands.append((w, pl, 0))
            if emulated:
                cands += [(w, False, sh) for sh in shares]
        table = []
        for w, pl, sh in cands:
            reg.SetSweepWidth(w)
            reg.SetSweepPipeline(pl)
            if emulated:
                reg.SetNativeShare(sh)
            _layer(reg, rng)
            reg.ApplyFusedGates()
            reg.synchronize()
            t = []
            for _ in range(trials):
                t0 = time.perf_counter()
                _layer(reg, rng)
                reg.ApplyFusedGates()
                reg.synchronize()
                t.append(time.perf_counter() - t0)
            table.append({"width": w, "pipeline": pl, "native_share": sh, "ms": 1e3 * min(t)})
        if not was:
            reg.TurnOffFusion()
        best = dict(min(table, key=lambda r: r["ms"]))
        best["table"] = table
        _CACHE[key] = best
    if apply:
        reg.SetSweepWidth(best["width"])
        reg.SetSweepPipeline(best["pipeline"])
        if emulated:
            reg.SetNativeShare(best["native_share"])
    return best


def cached(num_qubits: int, precision: str, math: int) -> Optional[dict]:
    return _CACHE.get((num_qubits, precision, math, _device_key()))
