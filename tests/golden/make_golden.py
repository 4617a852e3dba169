"""Generate tests/golden/golden.npz from the reference implementation itself.

Run in a checkout where the reference sources are available (IQS_REFERENCE_DIR, default
/root/reference); this builds oracle/_ref/libiqs_ref.so from those sources and drives the
reference's own QubitRegister<ComplexDP|ComplexSP> through oracle.RefRegister:

    python tests/golden/make_golden.py

Each case stores the operation list, its initial state, the final state (in full, or a
seeded sample of amplitudes for large registers), the final qubit map, and the values of
the query operations. The C restatement (oracle/iqs_oracle.c) and the GPU engine are both
checked against these vectors; neither is used to make them.
"""
from __future__ import annotations

import json
import math
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parents[1]
sys.path.insert(0, str(REPO))
sys.path.insert(0, str(REPO / "tests"))

import oracle  # noqa: E402
from circuits import dumps, enc, haar_2x2, plain_gate_by_gate, random_circuit, random_state, replay  # noqa: E402

FULL_STATE_MAX_QUBITS = 12
SAMPLE = 4096


def run_case(store: dict, name: str, n: int, ops: list, *, precision: str = "DP", init=None,
             style: str = "base", base: int = 0, fusion: int | None = None) -> None:
    ref = oracle.RefRegister(n, style, base, precision)
    if init is not None:
        ref.SetStateVector(init)
    if fusion is not None:
        ref.TurnOnFusion(fusion)
    q = replay(ref, ops)
    if fusion is not None:
        ref.TurnOffFusion()
    final = ref.GetStateVector().astype(np.complex128)
    meta = {"n": n, "precision": precision, "style": style, "base": base, "fusion": fusion}
    store[f"{name}/meta"] = np.array(json.dumps(meta))
    store[f"{name}/ops"] = np.array(dumps(ops))
    if init is not None:
        store[f"{name}/init"] = np.asarray(init, dtype=np.complex128)
    if n <= FULL_STATE_MAX_QUBITS:
        store[f"{name}/final"] = final
    else:
        rng = np.random.default_rng(1234)
        idx = np.sort(rng.choice(1 << n, size=SAMPLE, replace=False)).astype(np.int64)
        nz = np.flatnonzero(final)
        if nz.size <= SAMPLE:  # sparse state: keep every nonzero amplitude
            idx = np.union1d(idx, nz).astype(np.int64)
        store[f"{name}/final_idx"] = idx
        store[f"{name}/final"] = final[idx]
        store[f"{name}/final_norm2"] = np.array(float(np.vdot(final, final).real))
        store[f"{name}/final_sum4"] = np.array(float(np.sum(np.abs(final) ** 4)))
    store[f"{name}/map"] = np.asarray(ref.map, dtype=np.int64)
    store[f"{name}/queries"] = np.asarray(q, dtype=np.float64)
    print(f"{name:28s} n={n:2d} {precision} ops={len(ops):4d} queries={len(q)}")


def kat_cases(store: dict) -> None:
    # unit_test/include/apply_1q_gate_test.hpp: gates on qubit n-1 of a 4-qubit register, |0> and |8>
    for base in (0, 8):
        run_case(store, f"kat_1q_hadamard_{base}", 4, [["ApplyHadamard", [3]], ["ComputeNorm", []]], base=base)
        run_case(store, f"kat_1q_rx_{base}", 4, [["ApplyRotationX", [3, 0.83]]], base=base)
        run_case(store, f"kat_1q_ry_{base}", 4, [["ApplyRotationY", [3, 0.75]]], base=base)
        run_case(store, f"kat_1q_rz_{base}", 4, [["ApplyRotationZ", [3, 0.35]]], base=base)
        run_case(store, f"kat_1q_rxy_{base}", 4, [["ApplyRotationXY", [3, 0.4, 1.1]]], base=base)
    g = [[0.592056606032915 + 0.459533060553574j, -0.314948020757856 - 0.582328159830658j],
         [0.658235557641767 + 0.070882241549507j, 0.649564427121402 + 0.373855203932477j]]
    run_case(store, "kat_1q_custom", 4,
             [["Apply1QubitGate", [q, enc(g)]] for q in range(4)] + [["GetProbability", [q]] for q in range(4)],
             base=1 + 4)
    # unit_test/include/single_qubit_gates_test.hpp: Pauli operators and rotations on 10 qubits
    ops = [["ApplyPauliX", [0]], ["ApplyPauliY", [1]], ["ApplyPauliZ", [2]], ["ApplyRotationX", [3, math.pi]],
           ["ApplyPauliX", [3]]] + [["GetProbability", [q]] for q in range(10)]
    run_case(store, "kat_paulis_10q", 10, ops)
    # unit_test/include/apply_swap_gate_test.hpp: explicit 3-qubit example
    init = np.arange(8, dtype=np.complex128)
    run_case(store, "kat_swap_3q", 3, [["ApplySwap", [0, 1]], ["ApplySwap", [0, 1]], ["ApplySwap", [0, 2]]], init=init)
    # measure_test.hpp / expectation_values_test.hpp style: Bell and GHZ states
    ops = [["ApplyHadamard", [0]], ["ApplyCPauliX", [0, 1]], ["ApplyCPauliX", [1, 2]],
           ["GetProbability", [0]], ["GetProbability", [2]],
           ["ExpectationValue", [[0, 1], [3, 3], 1.0]], ["ExpectationValue", [[0, 1, 2], [1, 1, 1], 1.0]],
           ["ExpectationValue", [[0, 1, 2], [2, 2, 1], 1.0]], ["ExpectationValue", [[0], [1], 1.0]],
           ["ExpectationValue", [[2], [3], 2.0]], ["ExpectationValue", [[1, 2], [1, 2], 0.5]]]
    run_case(store, "kat_ghz_expect", 5, ops)
    # unit_test/include/qureg_permute_test.hpp: multi-cycle map on 20 qubits, sparse state
    n = 20
    vals = {2: 1, 8: 2, 1024: 3, 4096: 4, (1 << 19) + 512: 1j, (1 << 19) + 1024: 2j,
            (1 << 18) + 512: 3j, (1 << 18) + 1024: 4j}
    init = np.zeros(1 << n, dtype=np.complex128)
    for k, v in vals.items():
        init[k] = v
    mp = [4, 1, 2, 5, 6, 19, 16, 7, 10, 18, 8, 11, 12, 13, 14, 15, 0, 9, 17, 3]
    run_case(store, "kat_permute_20q", n, [["PermuteQubits", [mp, "direct"]], ["GetProbability", [5]]], init=init)
    mp2 = [1, 0, 2, 6, 4, 5, 3, 7, 8, 9, 12, 11, 10, 13, 14, 15, 16, 17, 18, 19]
    run_case(store, "kat_permute_local_20q", n,
             [["PermuteQubits", [mp2, "direct"]], ["PermuteQubits", [mp, "inverse"]]], init=init)


def random_cases(store: dict) -> None:
    specs = [(1, "DP", 11), (2, "DP", 12), (3, "DP", 13), (5, "DP", 14), (8, "DP", 15), (11, "DP", 16),
             (12, "DP", 17), (3, "SP", 21), (8, "SP", 22), (11, "SP", 23)]
    for n, prec, seed in specs:
        rng = np.random.default_rng(seed)
        init = random_state(n, rng)
        ops = random_circuit(n, 150, rng)
        run_case(store, f"random_{prec}_{n}q", n, ops, precision=prec, init=init)
    # Collapse + normalise (measurement with caller-supplied outcome).
    rng = np.random.default_rng(31)
    init = random_state(9, rng)
    ops = random_circuit(9, 40, rng, permutes=False) + [["CollapseQubit", [3, True]], ["ComputeNorm", []],
                                                         ["Normalize", []], ["GetProbability", [3]]]
    run_case(store, "collapse_DP_9q", 9, ops, init=init)
    # Fusion on: the reference replays buffered gates block by block; results must not change.
    # Apply2QubitGate is left out: it does not flush the reference's fusion buffer
    # (src/qureg_apply2qubitgate.cpp:14-73 never calls ApplyFusedGates), so buffered gates
    # would run after it, out of order.
    rng = np.random.default_rng(41)
    init = random_state(10, rng)
    ops = [o for o in random_circuit(10, 120, rng, permutes=False, queries=False) if o[0] != "Apply2QubitGate"]
    run_case(store, "fusion_DP_10q", 10, ops, init=init, fusion=4)


def config_cases(store: dict) -> None:
    # Plain gate-by-gate: 20 qubits, 20 layers of Haar U + CNOT bricks, from |0...0>.
    ops = plain_gate_by_gate(20, 20, seed=1)
    ops += [["ExpectationValue", [[0, 19], [3, 3], 1.0]], ["ComputeNorm", []]]
    run_case(store, "plain_gate_by_gate_20q", 20, ops)
    ops = plain_gate_by_gate(12, 20, seed=1)
    ops += [["ExpectationValue", [[0, 11], [3, 3], 1.0]], ["ComputeNorm", []]]
    run_case(store, "plain_gate_by_gate_12q", 12, ops)


def qaoa_cases(store: dict) -> None:
    """unit_test/include/qaoa_features_test.hpp: ring of 6 vertices, gamma 0.4, beta 0.3; and a
    seeded random graph on 10 vertices."""
    L = oracle.rlib()
    for name, n, adj, gammas, betas in (
            ("qaoa_ring6", 6, [[1 if abs(i - j) in (1, 5) else 0 for j in range(6)] for i in range(6)], [0.4], [0.3]),
            ("qaoa_random10", 10, None, [0.7, -0.3], [0.2, 0.45])):
        if adj is None:
            rng = np.random.default_rng(51)
            a = np.triu((rng.random((n, n)) < 0.4).astype(int), 1)
            adj = (a + a.T).tolist()
        flat = np.asarray(adj, dtype=np.int32).reshape(-1)
        diag = oracle.RefRegister(n, "base", 0)
        mx = L.ref_qaoa_maxcut_cost(diag.h, flat.ctypes.data_as(oracle._IP), n)
        psi = oracle.RefRegister(n, "++++", 0)
        for g, b in zip(gammas, betas):
            L.ref_qaoa_layer(psi.h, diag.h, g)
            for q in range(n):
                psi.ApplyRotationX(q, 2 * b)
        e1 = L.ref_qaoa_expectation(psi.h, diag.h)
        e2 = L.ref_qaoa_expectation_sq(psi.h, diag.h)
        store[f"{name}/meta"] = np.array(json.dumps({"n": n, "gammas": gammas, "betas": betas}))
        store[f"{name}/adjacency"] = flat.astype(np.int64)
        store[f"{name}/cost"] = diag.GetStateVector().real.copy()
        store[f"{name}/max_cut"] = np.array(mx)
        store[f"{name}/final"] = psi.GetStateVector()
        store[f"{name}/expectation"] = np.array([e1, e2])
        print(f"{name:28s} n={n:2d} max_cut={mx} <C>={e1:.6f}")


def main() -> None:
    oracle.build(ref=True)
    store: dict = {}
    kat_cases(store)
    random_cases(store)
    config_cases(store)
    qaoa_cases(store)
    out = HERE / "golden.npz"
    np.savez_compressed(out, **store)
    print(f"wrote {out} ({out.stat().st_size / 1e6:.2f} MB, {len(store)} arrays)")


if __name__ == "__main__":
    main()
