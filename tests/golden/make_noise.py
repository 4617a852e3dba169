"""Generate tests/golden/noise.npz from the reference itself, through oracle/ref_capi.cpp:

    python tests/golden/make_noise.py

- rng/*: draw sequences of the reference's RandomNumberGenerator<double|float>
  (src/rng_utils.cpp:13-225): uniforms, Gaussians, integers, skips and a copy, with final counts.
- noise/*: SetNoiseTimescales + ApplyNoiseGate (src/qureg_noisysimul.cpp:18-85) on seeded
  generators; the first case is the reference's unit test NoisySimulationTest.OneStateAtATime.
- noisy/*: NoisyQureg programs (include/NoisyQureg.hpp): states and experimental gate counts.
- chinorm/*: NormalizeEigenProbAndRenormalizeEigenVect (src/chi_matrix.cpp:166-200) on given
  eigensystems.
- channel/*: ApplyChannel (src/qureg_apply_channel.cpp:17-106) with given eigensystems, 1 and 2
  qubits, with negative eigenvalues; hadamard/*: the reference's IdealHadamard channel test.
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

_DP = C.POINTER(C.c_double)
_UP = C.POINTER(C.c_uint)
_IP = C.POINTER(C.c_int)

# (kind, n, stream): 0 uniform [0,1), 1 uniform [-2,5), 2 Gaussian, 3 integers [-3,17), 4 skip, 5 copy
RNG_OPS = [(0, 10, 2), (0, 5, 0), (2, 7, 1), (3, 9, 2), (4, 4, 1), (2, 3, 1), (5, 0, 0), (0, 6, 1), (2, 5, 2),
           (1, 4, 0), (4, 3, 2), (2, 1, 0), (0, 2, 0)]


def random_state(n, rng):
    v = rng.standard_normal(1 << n) + 1j * rng.standard_normal(1 << n)
    return v / np.linalg.norm(v)


def random_unitary(m, rng):
    z = rng.standard_normal((m, m)) + 1j * rng.standard_normal((m, m))
    q, r = np.linalg.qr(z)
    return q * (np.diag(r) / np.abs(np.diag(r)))


def set_state(reg, psi):
    a = np.ascontiguousarray(psi.astype(np.complex128)).view(np.float64)
    reg.L.ref_set_state(reg.h, a.ctypes.data_as(_DP))


def rng_cases(L, store):
    ops = np.array(RNG_OPS, dtype=np.int32).reshape(-1)
    for seed in (777, 717):
        for prec in ("DP", "SP"):
            out = np.zeros(256)
            counts = (C.c_ulong * 3)()
            k = L.ref_rng_sequence(1 if prec == "SP" else 0, seed, ops.ctypes.data_as(_IP), len(RNG_OPS),
                                   out.ctypes.data_as(_DP), len(out), counts)
            name = f"rng/{prec.lower()}_{seed}"
            store[f"{name}/meta"] = np.array(json.dumps({"seed": seed, "precision": prec, "ops": RNG_OPS}))
            store[f"{name}/values"] = out[:k].copy()
            store[f"{name}/counts"] = np.array(list(counts), dtype=np.uint64)


def noise_cases(L, store):
    rng = np.random.default_rng(31)
    cases = []
    # NoisySimulationTest.OneStateAtATime: |100111> (index 1+8+16+32), H on 0 and 1, T1=6, T2=4,
    # seed 7777, duration 5 on every qubit
    init = np.zeros(64, complex)
    init[1 + 8 + 16 + 32] = 1
    psi = init.reshape([2] * 6)
    for q in (0, 1):  # qubit q is bit q of the index: axis 5 - q
        ax = 5 - q
        psi = np.moveaxis(np.tensordot(np.array([[1, 1], [1, -1]]) / np.sqrt(2), np.moveaxis(psi, ax, 0), axes=1), 0, ax)
    cases.append(("unit_test_6q", 6, psi.reshape(-1), 7777, 6.0, 4.0, list(range(6)), [5.0] * 6))
    qs = [int(x) for x in rng.integers(0, 8, 24)]
    ds = [float(x) for x in rng.uniform(0.1, 3.0, 24)]
    ds[5] = 0.0  # no draw for a zero duration
    cases.append(("random_8q", 8, random_state(8, rng), 4242, 7.0, 4.0, qs, ds))
    cases.append(("dissipation_5q", 5, random_state(5, rng), 99, 6.0, 3.0, [0, 1, 2, 3, 4, 2], [6.0] * 6))
    for name, n, init, seed, T1, T2, qubits, durs in cases:
        for prec in ("DP", "SP"):
            r = oracle.RefRegister(n, "base", 0, prec)
            set_state(r, init)
            counts = (C.c_ulong * 3)()
            qa = np.array(qubits, dtype=np.uint32)
            da = np.array(durs, dtype=np.float64)
            L.ref_noise_run(r.h, seed, T1, T2, qa.ctypes.data_as(_UP), da.ctypes.data_as(_DP), len(qubits), counts)
            key = f"noise/{name}_{prec.lower()}"
            store[f"{key}/meta"] = np.array(json.dumps({"n": n, "precision": prec, "seed": seed, "T1": T1, "T2": T2,
                                                        "qubits": qubits, "durations": durs}))
            store[f"{key}/init"] = init.astype(np.complex128)
            store[f"{key}/state"] = r.GetStateVector().astype(np.complex128)
            store[f"{key}/counts"] = np.array(list(counts), dtype=np.uint64)


def noisy_cases(L, store):
    rng = np.random.default_rng(77)
    n = 5
    prog, angles, mats = [], [], []
    for i in range(40):
        kind = int(rng.integers(0, 8)) if i % 13 != 12 else 7
        a = int(rng.integers(0, n))
        b = int((a + 1 + rng.integers(0, n - 1)) % n)
        prog.append((kind, a, b))
        angles.append(float(rng.uniform(-np.pi, np.pi)))
        mats.append(random_unitary(2, rng).reshape(-1))
    prog_a = np.array(prog, dtype=np.int32).reshape(-1)
    ang_a = np.array(angles)
    mat_a = np.ascontiguousarray(np.array(mats, dtype=np.complex128)).view(np.float64).reshape(-1)
    for name, seed, T1, T2, Ts, Td in (("defaults", 12345, 2000.0, 1000.0, 1.0, 1.0),
                                       ("strong", 2024, 60.0, 40.0, 2.0, 5.0)):
        for prec in ("DP", "SP"):
            state = np.zeros(2 << n)
            counts = np.zeros(2 + n * n, dtype=np.uint32)
            L.ref_noisy_qureg_run(1 if prec == "SP" else 0, n, seed, T1, T2, Ts, Td, prog_a.ctypes.data_as(_IP),
                                  ang_a.ctypes.data_as(_DP), mat_a.ctypes.data_as(_DP), len(prog),
                                  state.ctypes.data_as(_DP), counts.ctypes.data_as(_UP))
            key = f"noisy/{name}_{prec.lower()}"
            store[f"{key}/meta"] = np.array(json.dumps({"n": n, "precision": prec, "seed": seed, "T1": T1, "T2": T2,
                                                        "Ts": Ts, "Td": Td, "prog": prog, "angles": angles}))
            store[f"{key}/mats"] = np.array(mats, dtype=np.complex128)
            store[f"{key}/state"] = state.view(np.complex128).copy()
            store[f"{key}/counts"] = counts


def eigensystem(m, evals, rng):
    u = random_unitary(m, rng)
    vecs = np.ascontiguousarray(u.T)  # row k = eigenvector k
    return np.asarray(evals, dtype=np.complex128), vecs


def chi_cases(L, store):
    rng = np.random.default_rng(5)
    systems = {
        "m4_mixed": eigensystem(4, [0.7, -0.1, 0.25, 0.05], rng),
        "m4_unit": eigensystem(4, [0.5, 0.25, 0.25, 0.0], rng),
        "m16_mixed": eigensystem(16, list(rng.uniform(-0.05, 0.3, 16)), rng),
    }
    for name, (ev, vecs) in systems.items():
        m = len(ev)
        for prec in ("DP", "SP"):
            evf = np.ascontiguousarray(ev).view(np.float64)
            vf = np.ascontiguousarray(vecs).view(np.float64).reshape(-1)
            probs, cum = np.zeros(m), np.zeros(m)
            out = np.zeros(2 * m * m)
            L.ref_chi_normalize(1 if prec == "SP" else 0, m, evf.ctypes.data_as(_DP), vf.ctypes.data_as(_DP),
                                probs.ctypes.data_as(_DP), cum.ctypes.data_as(_DP), out.ctypes.data_as(_DP))
            key = f"chinorm/{name}_{prec.lower()}"
            store[f"{key}/evals"] = ev
            store[f"{key}/evecs"] = vecs
            store[f"{key}/probs"] = probs
            store[f"{key}/cumprobs"] = cum
            store[f"{key}/vecs"] = out.view(np.complex128).reshape(m, m)
    # channels
    n = 5
    for name, steps in (("m4_mixed", 14), ("m16_mixed", 8)):
        ev, vecs = systems[name]
        m = len(ev)
        if m == 4:
            qubits = [int(x) for x in rng.integers(0, n, steps)]
        else:
            qubits = []
            for _ in range(steps):
                a, b = rng.choice(n, 2, replace=False)
                qubits += [int(a), int(b)]
        init = random_state(n, rng)
        for prec in ("DP", "SP"):
            r = oracle.RefRegister(n, "base", 0, prec)
            set_state(r, init)
            evf = np.ascontiguousarray(ev).view(np.float64)
            vf = np.ascontiguousarray(vecs).view(np.float64).reshape(-1)
            qa = np.array(qubits, dtype=np.uint32)
            sign = L.ref_channel_run(r.h, 3131, m, evf.ctypes.data_as(_DP), vf.ctypes.data_as(_DP),
                                     qa.ctypes.data_as(_UP), steps)
            key = f"channel/{name}_{prec.lower()}"
            store[f"{key}/meta"] = np.array(json.dumps({"n": n, "precision": prec, "seed": 3131, "qubits": qubits,
                                                        "steps": steps, "system": name}))
            store[f"{key}/init"] = init
            store[f"{key}/state"] = r.GetStateVector().astype(np.complex128)
            store[f"{key}/sign"] = np.array(sign)
    # ApplyQuantumChannel.IdealHadamard: |0100>, H on qubit 2, then the channel (seed 7777)
    for times in (1, 3):
        r = oracle.RefRegister(4, "base", 4, "DP")
        r.L.ref_named1(r.h, b"ApplyHadamard", 2, 0.0, 0.0)
        L.ref_ideal_hadamard_channel(r.h, 7777, 2, times)
        store[f"hadamard/times{times}/state"] = r.GetStateVector().astype(np.complex128)


def main() -> None:
    oracle.build(ref=True)
    L = oracle.rlib()
    store = {}
    rng_cases(L, store)
    noise_cases(L, store)
    noisy_cases(L, store)
    chi_cases(L, store)
    np.savez_compressed(HERE / "noise.npz", **store)
    print("wrote", len(store), "arrays:", sorted({"/".join(k.split("/")[:2]) for k in store}))


if __name__ == "__main__":
    main()
