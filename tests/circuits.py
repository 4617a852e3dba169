"""Seeded circuits and a replay loop shared by the golden-vector generator and the tests.

A circuit is a list of operations ``[name, args]`` where ``name`` is a QubitRegister method
of the reference API and ``args`` are JSON-friendly (matrices as [[re, im], ...] rows).
``replay`` calls the named methods on any backend with that API (the reference through
oracle.RefRegister, the C restatement through oracle.OracleRegister, the GPU engine through
iqs_gb300.QubitRegister) and collects the values returned by query operations.
"""
from __future__ import annotations

import json
import math
from typing import Any, List

import numpy as np

QUERIES = {"GetProbability", "ExpectationValue", "ComputeNorm"}


def haar_2x2(rng: np.random.Generator) -> np.ndarray:
    """Haar-random U(2): QR of a complex Gaussian matrix, phases of R's diagonal folded in."""
    z = (rng.standard_normal((2, 2)) + 1j * rng.standard_normal((2, 2))) / math.sqrt(2.0)
    q, r = np.linalg.qr(z)
    d = np.diag(r)
    return q * (d / np.abs(d))


def haar_4x4(rng: np.random.Generator) -> np.ndarray:
    z = (rng.standard_normal((4, 4)) + 1j * rng.standard_normal((4, 4))) / math.sqrt(2.0)
    q, r = np.linalg.qr(z)
    d = np.diag(r)
    return q * (d / np.abs(d))


def enc(m) -> list:
    a = np.asarray(m, dtype=np.complex128)
    return [[[float(x.real), float(x.imag)] for x in row] for row in a]


def dec(m) -> np.ndarray:
    return np.array([[complex(x[0], x[1]) for x in row] for row in m], dtype=np.complex128)


def _is_matrix(a) -> bool:
    return isinstance(a, list) and a and isinstance(a[0], list) and a[0] and isinstance(a[0][0], list)


def replay(reg, ops: List[list]) -> List[Any]:
    """Apply ops to reg; return the results of the query operations, in order."""
    results = []
    for name, args in ops:
        args = [dec(a) if _is_matrix(a) else a for a in args]
        r = getattr(reg, name)(*args)
        if name in QUERIES:
            results.append(float(r))
    return results


def random_state(n: int, rng: np.random.Generator) -> np.ndarray:
    v = rng.standard_normal(1 << n) + 1j * rng.standard_normal(1 << n)
    return (v / np.linalg.norm(v)).astype(np.complex128)


def random_circuit(n: int, num_ops: int, rng: np.random.Generator, *, permutes: bool = True,
                   queries: bool = True) -> List[list]:
    """A mix of every gate family of the hot path on random qubits and parameters."""
    ops: List[list] = []
    one_named = ["ApplyPauliX", "ApplyPauliY", "ApplyPauliZ", "ApplyPauliSqrtX", "ApplyPauliSqrtY",
                 "ApplyPauliSqrtZ", "ApplyT", "ApplyHadamard"]
    one_rot = ["ApplyRotationX", "ApplyRotationY", "ApplyRotationZ"]
    two_named = ["ApplyCPauliX", "ApplyCPauliY", "ApplyCPauliZ", "ApplyCPauliSqrtZ", "ApplyCHadamard"]
    two_rot = ["ApplyCRotationX", "ApplyCRotationY", "ApplyCRotationZ", "ApplyCPhaseRotation"]
    swaps = ["ApplySwap", "ApplyISwap", "ApplySqrtISwap", "Apply4thRootISwap"]

    def q():
        return int(rng.integers(n))

    def two():
        a, b = rng.choice(n, size=2, replace=False)
        return int(a), int(b)

    def ang():
        return float(rng.uniform(-math.pi, math.pi))

    kinds = ["u1", "named1", "rot1", "rxy"]
    if n >= 2:
        kinds += ["u1c", "named2", "rot2", "swap", "iswaprot", "u2", "diag"]
    if n >= 3:
        kinds += ["toffoli"]
    if permutes and n >= 2:
        kinds += ["permute", "emulate"]
    if queries:
        kinds += ["prob", "expect", "norm"]
    # Track the qubit -> position map: the reference's Apply2QubitGate picks its loop order
    # from the qubit order but its strides from the positions, and indexes past the end of
    # the state when the two orders disagree (src/qureg_apply2qubitgate.cpp:41-64). Those
    # cases are left out of the circuits the reference runs.
    qmap = list(range(n))
    for _ in range(num_ops):
        k = kinds[int(rng.integers(len(kinds)))]
        if k == "u2":
            a, b = two()
            if (a > b) != (qmap[a] > qmap[b]):
                k = "u1c"
        if k == "u1":
            ops.append(["Apply1QubitGate", [q(), enc(haar_2x2(rng))]])
        elif k == "named1":
            ops.append([one_named[int(rng.integers(len(one_named)))], [q()]])
        elif k == "rot1":
            ops.append([one_rot[int(rng.integers(len(one_rot)))], [q(), ang()]])
        elif k == "rxy":
            ops.append(["ApplyRotationXY", [q(), ang(), ang()]])
        elif k == "u1c":
            a, b = two()
            ops.append(["ApplyControlled1QubitGate", [a, b, enc(haar_2x2(rng))]])
        elif k == "named2":
            a, b = two()
            ops.append([two_named[int(rng.integers(len(two_named)))], [a, b]])
        elif k == "rot2":
            a, b = two()
            ops.append([two_rot[int(rng.integers(len(two_rot)))], [a, b, ang()]])
        elif k == "swap":
            a, b = two()
            ops.append([swaps[int(rng.integers(len(swaps)))], [a, b]])
        elif k == "iswaprot":
            a, b = two()
            u = haar_2x2(rng)
            m = np.array([[u[0, 0], u[0, 1]], [u[0, 1], u[1, 1]]])  # symmetric off-diagonal
            ops.append(["ApplyISwapRotation", [a, b, enc(m)]])
        elif k == "u2":
            ops.append(["Apply2QubitGate", [a, b, enc(haar_4x4(rng))]])
        elif k == "diag":
            a, b = two()
            ph = rng.uniform(-math.pi, math.pi, 4)
            ops.append(["ApplyDiag", [a, b, enc(np.diag(np.exp(1j * ph)))]])
        elif k == "toffoli":
            a, b, c = (int(x) for x in rng.choice(n, size=3, replace=False))
            ops.append(["ApplyToffoli", [a, b, c]])
        elif k == "permute":
            qmap = [int(x) for x in rng.permutation(n)]
            ops.append(["PermuteQubits", [list(qmap), "direct"]])
        elif k == "emulate":
            a, b = two()
            qmap[a], qmap[b] = qmap[b], qmap[a]
            ops.append(["EmulateSwap", [a, b]])
        elif k == "prob":
            ops.append(["GetProbability", [q()]])
        elif k == "expect":
            kq = int(rng.integers(1, min(n, 4) + 1))
            qs = [int(x) for x in rng.choice(n, size=kq, replace=False)]
            obs = [int(x) for x in rng.integers(1, 4, size=kq)]
            ops.append(["ExpectationValue", [qs, obs, float(rng.uniform(0.5, 2.0))]])
        elif k == "norm":
            ops.append(["ComputeNorm", []])
    return ops


def brick_layer_ops(n: int, rng: np.random.Generator, entangler: str = "ApplyCPauliX") -> List[list]:
    """One layer: a Haar U on every qubit, then the entangler on even pairs, then odd pairs."""
    ops = [["Apply1QubitGate", [q, enc(haar_2x2(rng))]] for q in range(n)]
    ops += [[entangler, [2 * j, 2 * j + 1]] for j in range(n // 2)]
    ops += [[entangler, [2 * j + 1, 2 * j + 2]] for j in range((n - 1) // 2)]
    return ops


def plain_gate_by_gate(n: int = 20, layers: int = 20, seed: int = 1) -> List[list]:
    """The 20-qubit, 20-layer Haar + CNOT-brick circuit (780 gates at n = 20)."""
    rng = np.random.default_rng(seed)
    ops: List[list] = []
    for _ in range(layers):
        ops += brick_layer_ops(n, rng, "ApplyCPauliX")
    return ops


def qft_ops(n: int) -> List[list]:
    """Quantum Fourier transform in the gate order of examples/quantum_fourier_transform.cpp:49-71:
    for i = n-1..0, controlled phase diag(1, e^{i pi / 2^(j-i)}) with control j > i (from n-1
    down) on target i, then H(i); then SWAP(i, n-1-i) for i < n/2."""
    ops: List[list] = []
    for i in range(n - 1, -1, -1):
        for j in range(n - 1, i, -1):
            ph = math.pi / float(1 << (j - i))
            ops.append(["ApplyControlled1QubitGate", [j, i, enc([[1, 0], [0, complex(math.cos(ph), math.sin(ph))]])]])
        ops.append(["ApplyHadamard", [i]])
    for i in range(n // 2):
        ops.append(["ApplySwap", [i, n - 1 - i]])
    return ops


def qft_brick(n: int = 30, layers: int = 40, seed: int = 2) -> List[list]:
    """QFT followed by `layers` layers of (Haar U on every qubit + CZ brick, even then odd)."""
    rng = np.random.default_rng(seed)
    ops = qft_ops(n)
    for _ in range(layers):
        ops += brick_layer_ops(n, rng, "ApplyCPauliZ")
    return ops


def qft_brick_start(n: int, seed: int = 2) -> int:
    """Basis state the QFT + brick circuit starts from (a QFT of |0...0> would be trivial)."""
    return int(np.random.default_rng(seed + 1000).integers(1 << n))


def qft_brick_queries(n: int) -> List[list]:
    """Queries read after the QFT + brick circuit."""
    return [["ComputeNorm", []], ["GetProbability", [0]], ["GetProbability", [n - 1]],
            ["ExpectationValue", [[0, n - 1], [3, 3], 1.0]]]


def dumps(ops) -> str:
    return json.dumps(ops, separators=(",", ":"))


def loads(s: str) -> List[list]:
    return json.loads(s)
