"""Generate tests/golden/qaoa_extra.npz from the reference itself: the weighted MaxCut cost
vector and the three cost histograms (src/qaoa_features.cpp:153-538), run through the
reference's own QubitRegister and iqs::qaoa functions (oracle.RefRegister and
oracle/ref_capi.cpp; the reference is built from its sources by oracle/Makefile):

    python tests/golden/make_qaoa_extra.py

Cases: the weighted ring of 6 from unit_test/include/qaoa_features_test.hpp (vertical edges
1.4; gamma 0.4, beta 0.3; rounded histogram and bins of 0.1), the unweighted ring of 6 with
its integer histogram, and a seeded weighted graph on 10 vertices (two layers; bins of 0.25)
in ComplexDP, and its cost vector and state in ComplexSP. Each case keeps the adjacency, the angles, the full cost vector,
the maximum, the final state, the expectation and the histograms.
"""
from __future__ import annotations

import ctypes as C
import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parents[1]
sys.path.insert(0, str(REPO))

import oracle  # noqa: E402


def run(L, name, n, adj, gammas, betas, prec, weighted, hists, store):
    diag = oracle.RefRegister(n, "base", 0, prec)
    psi = oracle.RefRegister(n, "++++", 0, prec)
    flat = np.ascontiguousarray(np.asarray(adj, dtype=np.float64).reshape(-1))
    if weighted:
        mx = L.ref_qaoa_weighted_cost(diag.h, flat.ctypes.data_as(oracle._DP), n)
    else:
        iflat = np.ascontiguousarray(flat.astype(np.int32))
        mx = float(L.ref_qaoa_maxcut_cost(diag.h, iflat.ctypes.data_as(oracle._IP), n))
    for g, b in zip(gammas, betas):
        L.ref_qaoa_layer(psi.h, diag.h, g)
        for q in range(n):
            psi.ApplyRotationX(q, b)
    e = L.ref_qaoa_expectation(psi.h, diag.h)
    meta = {"n": n, "precision": prec, "weighted": weighted, "gammas": gammas, "betas": betas, "max_cut": mx,
            "expectation": e, "hists": hists}
    store[f"{name}/meta"] = np.array(json.dumps(meta))
    store[f"{name}/adj"] = flat
    store[f"{name}/diag"] = diag.GetStateVector().astype(np.complex128)
    store[f"{name}/psi"] = psi.GetStateVector().astype(np.complex128)
    for k, (mode, width) in enumerate(hists):
        out = np.zeros(4096)
        ln = L.ref_qaoa_histogram(psi.h, diag.h, mode, mx, width, out.ctypes.data_as(oracle._DP), out.size)
        store[f"{name}/hist{k}"] = out[:ln].copy()


def main() -> None:
    oracle.build(ref=True)
    L = oracle.rlib()
    store = {}
    w6 = [[0, 1, 0, 0, 0, 1.4], [1, 0, 1, 0, 0, 0], [0, 1, 0, 1.4, 0, 0],
          [0, 0, 1.4, 0, 1, 0], [0, 0, 0, 1, 0, 1], [1.4, 0, 0, 0, 1, 0]]
    run(L, "w_ring6", 6, w6, [0.4], [0.3], "DP", True, [(1, 1.0), (2, 0.1)], store)
    r6 = [[1 if abs(i - j) in (1, 5) else 0 for j in range(6)] for i in range(6)]
    run(L, "ring6", 6, r6, [0.4], [0.3], "DP", False, [(0, 1.0)], store)
    rng = np.random.default_rng(17)
    n = 10
    a = np.zeros((n, n))
    for i in range(n):
        for j in range(i + 1, n):
            if rng.random() < 0.5:
                a[i, j] = a[j, i] = round(float(rng.uniform(0.5, 2.0)), 3)
    run(L, "w_random10_DP", n, a.tolist(), [0.35, -0.6], [0.25, 0.4], "DP", True, [(1, 1.0), (2, 0.25)], store)
    # In ComplexSP the reference's float cost formula leaves some cut values slightly below
    # -1e-7 and its weighted histograms abort on their range assert, so the SP case keeps the
    # cost vector and the state only.
    run(L, "w_random10_SP", n, a.tolist(), [0.35, -0.6], [0.25, 0.4], "SP", True, [], store)
    np.savez_compressed(HERE / "qaoa_extra.npz", **store)
    print("wrote", sorted({k.split('/')[0] for k in store}))


if __name__ == "__main__":
    main()
