"""The C++ drop-in header include/iqs_gb300/qureg.hpp: a driver written against
iqs::QubitRegister<ComplexDP> (tests/cpp/shim_driver.cpp) runs a seeded circuit on the GPU,
with and without fusion; its state, query results, gate count and qubit map are compared
with the oracle running the same gates."""
import subprocess

import numpy as np
import pytest

import oracle
from conftest import REPO, TOL_DP

pytestmark = pytest.mark.gpu


def _circuit(n, rng, fusion):
    lines, ops = [f"{n}"], []
    if fusion:
        lines.append("FUSION on")

    def u2():
        z = rng.standard_normal((2, 2)) + 1j * rng.standard_normal((2, 2))
        q, _ = np.linalg.qr(z)
        return q

    for layer in range(4):
        for q in range(n):
            m = u2()
            lines.append("U1 %d " % q + " ".join(f"{float(x.real)!r} {float(x.imag)!r}" for x in m.reshape(-1)))
            ops.append(("Apply1QubitGate", (q, m)))
        for q in range(layer % 2, n - 1, 2):
            lines.append(f"CNOT {q} {q + 1}")
            ops.append(("ApplyCPauliX", (q, q + 1)))
        t = float(rng.uniform(-3, 3))
        lines.append(f"CPHASE {layer} {n - 1 - layer} {t!r}")
        ops.append(("ApplyCPhaseRotation", (layer, n - 1 - layer, t)))
    m = u2()
    lines.append("CU1 2 5 " + " ".join(f"{float(x.real)!r} {float(x.imag)!r}" for x in m.reshape(-1)))
    ops.append(("ApplyControlled1QubitGate", (2, 5, m)))
    z = rng.standard_normal((4, 4)) + 1j * rng.standard_normal((4, 4))
    m4, _ = np.linalg.qr(z)
    lines.append("U2 6 1 " + " ".join(f"{float(x.real)!r} {float(x.imag)!r}" for x in m4.reshape(-1)))
    ops.append(("Apply2QubitGate", (6, 1, m4)))
    for name, code, args in (("ApplyToffoli", "TOFFOLI", (0, 3, 7)), ("ApplySwap", "SWAP", (1, 8)),
                             ("ApplyISwap", "ISWAP", (4, 2)), ("ApplyRotationXY", "RXY", (3, 0.4, 1.3)),
                             ("ApplyT", "T", (9,)), ("ApplyPauliY", "Y", (5,))):
        lines.append(code + " " + " ".join(repr(a) for a in args))
        ops.append((name, args))
    perm = [int(x) for x in rng.permutation(n)]
    lines.append("PERM " + " ".join(map(str, perm)))
    ops.append(("PermuteQubits", (perm,)))
    lines.append("H 4")
    ops.append(("ApplyHadamard", (4,)))
    queries = [("PROB 3", ("GetProbability", (3,))), ("EXPECT 2 0 9 3 3 1.5", ("ExpectationValue", ([0, 9], [3, 3], 1.5))),
               ("EXPECT 1 4 1 1.0", ("ExpectationValue", ([4], [1], 1.0))), ("NORM", ("ComputeNorm", ()))]
    return lines, ops, queries


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    d = tmp_path_factory.mktemp("shim")
    exe = d / "shim_driver"
    libdir = REPO / "intel-qs_gb300" / "iqs_gb300"
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", str(REPO / "include"), str(REPO / "tests" / "cpp" / "shim_driver.cpp"),
                    "-L", str(libdir), "-liqsg", f"-Wl,-rpath,{libdir}", "-o", str(exe)], check=True)
    return exe


@pytest.mark.parametrize("fusion", [False, True])
def test_cpp_header_matches_oracle(driver, tmp_path, fusion):
    n = 10
    rng = np.random.default_rng(811)
    lines, ops, queries = _circuit(n, rng, fusion)
    lines += [q[0] for q in queries]
    (tmp_path / "ops.txt").write_text("\n".join(lines) + "\n")
    subprocess.run([str(driver), str(tmp_path / "ops.txt"), str(tmp_path / "q.txt"), str(tmp_path / "s.bin")],
                   check=True)
    ref = oracle.OracleRegister(n, "base", 0)
    for name, args in ops:
        getattr(ref, name)(*args)
    expected_q = [getattr(ref, q[1][0])(*q[1][1]) for q in queries]
    out = (tmp_path / "q.txt").read_text().split("\n")
    got_q = [float(x) for x in out[:len(queries)]]
    assert np.max(np.abs(np.asarray(got_q) - np.asarray(expected_q))) <= TOL_DP
    gates = out[len(queries)].split()
    # 4 layers of n U1 and n - 1 CNOT, 4 CPHASE, CU1 + U2, Toffoli = 5 two-qubit gates, SWAP,
    # ISWAP, RXY, T, Y, H, and the X-basis change of EXPECT (applied and undone) = 2
    assert gates[0] == "gates" and int(gates[1]) == 4 * n + 2 * (n - 1) + 4 + 2 + 5 + 5 + 1 + 2
    maps = [int(l.split()[1]) for l in out if l.startswith("map ")]
    assert maps == ref.perm.map
    state = np.fromfile(tmp_path / "s.bin", dtype=np.complex128)
    assert np.max(np.abs(state - ref.GetStateVector())) <= TOL_DP
