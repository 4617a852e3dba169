"""Generate tests/golden/qft_brick.npz: the QFT + Haar/CZ-brick circuit run by the reference
itself (oracle.RefRegister over the reference's own QubitRegister<ComplexDP>).

    python tests/golden/make_qft_brick.py            # n = 24 and n = 30 (about 15 min on 8 cores)

For each n the file keeps the operation list itself (LAPACK and libm differ in the last bit
between machines, so a list regenerated elsewhere is not the same circuit), its generator
arguments and SHA-256, the start basis index, a seeded sample of 4096 final amplitudes, and
the values of the final queries (norm, P(q = 1) for two qubits, <Z_0 Z_{n-1}>).

    python tests/golden/make_qft_brick.py --ops-only   # add the operation lists of the
                                                       # stored cases (same machine only)
"""
from __future__ import annotations

import hashlib
import json
import os
import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parents[1]
sys.path.insert(0, str(REPO))
sys.path.insert(0, str(REPO / "tests"))

import oracle  # noqa: E402
from circuits import dumps, qft_brick, qft_brick_queries, qft_brick_start, replay  # noqa: E402

SAMPLE = 4096
LAYERS = 40
SEED = 2


def sample_index(n: int) -> np.ndarray:
    rng = np.random.default_rng(4321 + n)
    return np.sort(rng.choice(1 << n, size=SAMPLE, replace=False)).astype(np.int64)


def ops_hash(ops) -> str:
    return hashlib.sha256(dumps(ops).encode()).hexdigest()


def main(sizes=(24, 30)) -> None:
    oracle.build(ref=True)
    out = HERE / "qft_brick.npz"
    store = dict(np.load(out)) if out.exists() else {}
    for n in sizes:
        t0 = time.time()
        ops = qft_brick(n, LAYERS, SEED)
        start = qft_brick_start(n, SEED)
        ref = oracle.RefRegister(n, "base", start, "DP")
        replay(ref, ops)
        vals = replay(ref, qft_brick_queries(n))
        st = ref.GetStateVector()
        idx = sample_index(n)
        store[f"n{n}/meta"] = np.array(json.dumps({"n": n, "layers": LAYERS, "seed": SEED, "start": start,
                                                   "gates": len(ops), "ops_sha256": ops_hash(ops)}))
        store[f"n{n}/ops"] = np.array(dumps(ops))
        store[f"n{n}/idx"] = idx
        store[f"n{n}/amps"] = st[idx].astype(np.complex128)
        store[f"n{n}/queries"] = np.asarray(vals, dtype=np.float64)
        del ref, st
        print(f"n={n}: {len(ops)} gates in {time.time() - t0:.1f} s", flush=True)
        np.savez_compressed(out, **store)


def add_ops() -> None:
    out = HERE / "qft_brick.npz"
    store = dict(np.load(out))
    for key in [k for k in store if k.endswith("/meta")]:
        meta = json.loads(str(store[key]))
        ops = qft_brick(meta["n"], meta["layers"], meta["seed"])
        if ops_hash(ops) != meta["ops_sha256"]:
            raise SystemExit(f"{key}: the circuit generated here is not the one the amplitudes came from")
        store[key.replace("/meta", "/ops")] = np.array(dumps(ops))
    np.savez_compressed(out, **store)


if __name__ == "__main__":
    if sys.argv[1:] == ["--ops-only"]:
        add_ops()
    else:
        main(tuple(int(a) for a in sys.argv[1:]) or (24, 30))
