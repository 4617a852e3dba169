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


def test_cpp_qaoa_header_and_formats(tmp_path, capsys):
    """include/iqs_gb300/qaoa_features.hpp and the statistics / Print of the C++ register
    against the reference's outputs (tests/golden/qaoa_extra.npz) and the oracle."""
    import json
    import iqs_gb300 as iqs
    libdir = REPO / "intel-qs_gb300" / "iqs_gb300"
    exe = tmp_path / "qaoa_driver"
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", str(REPO / "include"), str(REPO / "tests" / "cpp" / "qaoa_driver.cpp"),
                    "-L", str(libdir), "-liqsg", f"-Wl,-rpath,{libdir}", "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, check=True)
    vals = {}
    text = []
    for line in r.stdout.splitlines():
        parts = line.split(" ")
        if len(parts) == 2 and parts[0] in ("max", "cost4", "cost36", "expect", "h0", "h1", "h2", "stat"):
            vals.setdefault(parts[0], []).append(float(parts[1]))
        else:
            text.append(line)
    z = np.load(REPO / "tests" / "golden" / "qaoa_extra.npz")
    meta = json.loads(str(z["w_ring6/meta"]))
    assert abs(vals["max"][0] - meta["max_cut"]) <= 1e-12
    assert abs(vals["cost4"][0] - 2.4) <= 1e-12 and abs(vals["cost36"][0] - 4.8) <= 1e-12
    assert abs(vals["expect"][0] - meta["expectation"]) <= 1e-12
    assert np.max(np.abs(np.asarray(vals["h1"]) - z["w_ring6/hist0"])) <= 1e-12
    assert np.max(np.abs(np.asarray(vals["h2"]) - z["w_ring6/hist1"])) <= 1e-12
    o = oracle.OracleRegister(6, "", 0)
    o.SetStateVector(z["w_ring6/psi"])
    assert np.max(np.abs(np.asarray(vals["stat"]) - oracle.oracle_google_stats(o)) /
                  np.maximum(1.0, np.abs(oracle.oracle_google_stats(o)))) <= 1e-12
    ring = [[1 if abs(i - j) in (1, 5) else 0 for j in range(6)] for i in range(6)]
    d = oracle.OracleRegister(6, "base", 0)
    m2 = oracle.oracle_maxcut_cost(d, np.asarray(ring, dtype=np.int32))
    assert np.max(np.abs(np.asarray(vals["h0"]) - oracle.oracle_cost_histogram(o, d, 0, m2))) <= 1e-12
    small = iqs.QubitRegister(2, "base", 2)
    small.ApplyHadamard(0)
    small.Print("small")
    assert "\n".join(text) + "\n" == capsys.readouterr().out
