"""Generate tests/golden/rand_init.npz from the reference itself: Initialize("rand") states
(src/qureg_init.cpp:253-330) of the reference's QubitRegister with its RandomNumberGenerator
(src/rng_utils.cpp), through oracle.RefRegister and oracle/ref_capi.cpp:

    python tests/golden/make_rand_init.py

Cases use the seeds of the reference's unit tests; one case initialises twice in a row (the
second state comes from the advanced stream), one uses the "local" stream (base_index 1).
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parents[1]
sys.path.insert(0, str(REPO))

import oracle  # noqa: E402

CASES = [("dp6_777", 6, "DP", 777, 0, 1), ("dp10_12345_twice", 10, "DP", 12345, 0, 2),
         ("sp8_7315", 8, "SP", 7315, 0, 1), ("dp5_7777_local", 5, "DP", 7777, 1, 1)]


def main() -> None:
    oracle.build(ref=True)
    L = oracle.rlib()
    store = {}
    for name, n, prec, seed, base, times in CASES:
        r = oracle.RefRegister(n, "base", 0, prec)
        L.ref_init_rand(r.h, seed, base, times)
        store[f"{name}/meta"] = np.array(json.dumps({"n": n, "precision": prec, "seed": seed, "base_index": base,
                                                     "times": times}))
        store[f"{name}/state"] = r.GetStateVector().astype(np.complex128)
    np.savez_compressed(HERE / "rand_init.npz", **store)
    print("wrote", sorted({k.split('/')[0] for k in store}))


if __name__ == "__main__":
    main()
