"""Generate tests/golden/state_io.npz from the reference itself: Entropy, GoogleStats, the
text of Print and of ExportAmplitudes (src/qureg_utils.cpp:303-657) for seeded states,
through the reference's own QubitRegister (oracle.RefRegister over oracle/ref_capi.cpp):

    python tests/golden/make_state_io.py

Cases: a 5-qubit ComplexDP state, the same state after a qubit permutation, and a 4-qubit
ComplexSP state. Print writes to the process's standard output; it is captured from file
descriptor 1.
"""
from __future__ import annotations

import ctypes as C
import json
import os
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parents[1]
sys.path.insert(0, str(REPO))

import oracle  # noqa: E402


def capture_fd1(fn) -> str:
    libc = C.CDLL(None)
    sys.stdout.flush()
    with tempfile.TemporaryFile(mode="w+b") as tmp:
        saved = os.dup(1)
        os.dup2(tmp.fileno(), 1)
        try:
            fn()
            libc.fflush(None)
        finally:
            os.dup2(saved, 1)
            os.close(saved)
        tmp.seek(0)
        return tmp.read().decode()


def case(L, store, name, n, prec, state, perm=None):
    r = oracle.RefRegister(n, "base", 0, prec)
    r.SetStateVector(state)
    if perm is not None:
        r.PermuteQubits(perm, "direct")
    stats = np.zeros(32)
    k = L.ref_google_stats(r.h, stats.ctypes.data_as(oracle._DP), 32)
    text = capture_fd1(lambda: L.ref_print(r.h, name.encode()))
    with tempfile.TemporaryDirectory() as d:
        f = os.path.join(d, "amps.json")
        L.ref_export(r.h, f.encode())
        export = open(f).read()
    store[f"{name}/meta"] = np.array(json.dumps({"n": n, "precision": prec, "perm": perm, "entropy": L.ref_entropy(r.h)}))
    store[f"{name}/init"] = np.asarray(state, dtype=np.complex128)
    store[f"{name}/stats"] = stats[:k].copy()
    store[f"{name}/print"] = np.array(text)
    store[f"{name}/export"] = np.array(export)


def main() -> None:
    oracle.build(ref=True)
    L = oracle.rlib()
    rng = np.random.default_rng(29)
    store = {}
    v = rng.standard_normal(32) + 1j * rng.standard_normal(32)
    v /= np.linalg.norm(v)
    v[3] = 0.0  # a zero amplitude: skipped by the entropy sums
    v /= np.linalg.norm(v)
    case(L, store, "dp5", 5, "DP", v)
    case(L, store, "dp5_perm", 5, "DP", v, [2, 0, 4, 1, 3])
    w = rng.standard_normal(16) + 1j * rng.standard_normal(16)
    w /= np.linalg.norm(w)
    case(L, store, "sp4", 4, "SP", w)
    np.savez_compressed(HERE / "state_io.npz", **store)
    print("wrote", sorted({k.split('/')[0] for k in store}))


if __name__ == "__main__":
    main()
