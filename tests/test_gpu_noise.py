"""Noise paths on the GPU against the reference's own trajectories (tests/golden/noise.npz, made
by tests/golden/make_noise.py): ApplyNoiseGate with seeded generators, NoisyQureg programs,
ApplyChannel on one and two qubits, and the reference's channel unit tests."""
import json

import numpy as np
import pytest

from conftest import REPO

pytestmark = pytest.mark.gpu

FIX = REPO / "tests" / "golden" / "noise.npz"
TOL = {"DP": 1e-13, "SP": 3e-6}


def _groups(prefix):
    z = np.load(FIX)
    return sorted({"/".join(k.split("/")[:2]) for k in z.files if k.startswith(prefix + "/")})


@pytest.mark.parametrize("key", _groups("noise"))
def test_noise_gates_match_reference(key):
    """SetNoiseTimescales + ApplyNoiseGate (src/qureg_noisysimul.cpp:18-85); the unit_test_6q case
    is NoisySimulationTest.OneStateAtATime (unit_test/include/noisy_simulation_test.hpp:58-84)."""
    import iqs_gb300 as iqs
    z = np.load(FIX)
    meta = json.loads(str(z[f"{key}/meta"]))
    prec = meta["precision"]
    r = iqs.QubitRegister(meta["n"], "base", 0, precision=prec)
    r.SetStateVector(z[f"{key}/init"])
    clean = iqs.QubitRegister(r)
    r.SetNoiseTimescales(meta["T1"], meta["T2"])
    rng = iqs.RandomNumberGenerator(precision=prec)
    rng.SetSeedStreamPtrs(meta["seed"])
    r.SetRngPtr(rng)
    for q, d in zip(meta["qubits"], meta["durations"]):
        r.ApplyNoiseGate(q, d)
    assert np.max(np.abs(r.GetStateVector() - z[f"{key}/state"])) <= TOL[prec]
    assert [rng.GetNumGeneratedOrSkippedPoolNumbers(), rng.GetNumGeneratedOrSkippedStateNumbers(),
            rng.GetNumGeneratedOrSkippedLocalNumbers()] == [int(x) for x in z[f"{key}/counts"]]
    assert r.ComputeOverlap(clean).real < 1 - 1e-15
    assert abs(r.ComputeNorm() - 1) <= TOL[prec] * 10


def test_noise_gate_checks():
    import iqs_gb300 as iqs
    r = iqs.QubitRegister(3, "base", 0)
    with pytest.raises(ValueError):  # no generator
        r.ApplyNoiseGate(0, 1.0)
    rng = iqs.RandomNumberGenerator()
    rng.SetSeedStreamPtrs(5)
    r.SetRngPtr(rng)
    with pytest.raises(ValueError):  # no timescales
        r.ApplyNoiseGate(0, 1.0)
    with pytest.raises(ValueError):  # T2 < T1/2, which the reference asserts against
        r.SetNoiseTimescales(6.0, 2.0)
    r.SetNoiseTimescales(6.0, 3.0)
    assert (r.GetT1(), r.GetT2()) == (6.0, 3.0) and r.GetTphi() == float("inf")
    r.SetNoiseTimescales(6.0, 4.0)
    assert abs(r.GetTphi() - 1 / (1 / 4 - 1 / 12)) < 1e-12
    before = r.GetStateVector()
    r.ApplyNoiseGate(1, 0.0)  # zero duration: no gate, no draw
    assert np.array_equal(r.GetStateVector(), before) and rng.GetNumGeneratedOrSkippedStateNumbers() == 0


def test_pure_dissipation_raises_ground_population():
    """NoisySimulationTest.TwoStates (noisy_simulation_test.hpp:88-129) for the state |0...0> of a
    one-state pool: pure dissipation (T2 = T1/2) for T1 on every qubit."""
    import iqs_gb300 as iqs
    psi = iqs.QubitRegister(6, "base", 0)
    rng = iqs.RandomNumberGenerator()
    rng.SetSeedStreamPtrs(7777)
    psi.SetRngPtr(rng)
    psi.SetNoiseTimescales(6.0, 3.0)
    for q in range(6):
        psi.ApplyNoiseGate(q, 6.0)
    assert psi.GetProbability(0) > 1e-15


@pytest.mark.parametrize("key", _groups("noisy"))
def test_noisy_qureg_matches_reference(key):
    """NoisyQureg (include/NoisyQureg.hpp): noise gates before each logical gate, its own
    std::default_random_engine, experimental gate counts."""
    import iqs_gb300 as iqs
    z = np.load(FIX)
    meta = json.loads(str(z[f"{key}/meta"]))
    prec, n = meta["precision"], meta["n"]
    r = iqs.NoisyQureg(n, meta["seed"], meta["T1"], meta["T2"], precision=prec)
    r.Initialize("base", 0)
    r.SetGateDurations(meta["Ts"], meta["Td"])
    mats = z[f"{key}/mats"]
    for i, (kind, a, b) in enumerate(meta["prog"]):
        ang = meta["angles"][i]
        m = mats[i].reshape(2, 2)
        if kind == 0:
            r.ApplyHadamard(a)
        elif kind == 1:
            r.ApplyRotationX(a, ang)
        elif kind == 2:
            r.ApplyRotationY(a, ang)
        elif kind == 3:
            r.ApplyRotationZ(a, ang)
        elif kind == 4:
            r.ApplyCPauliX(a, b)
        elif kind == 5:
            r.ApplyControlled1QubitGate(a, b, m)
        elif kind == 6:
            r.Apply1QubitGate(a, m)
        elif kind == 7:
            r.ApplyNoiseGatesOnAllQubits()
    assert np.max(np.abs(r.GetStateVector() - z[f"{key}/state"])) <= TOL[prec] * 10
    counts = z[f"{key}/counts"]
    assert r.GetOneQubitExperimentalGateCount() == counts[0]
    assert r.GetTwoQubitExperimentalGateCount() == counts[1]
    assert r.GetTotalExperimentalGateCount() == counts[0] + counts[1]
    got = np.array([r.GetExperimentalGateCount(x, y) for x in range(n) for y in range(n)])
    assert np.array_equal(got, counts[2:])
    assert r.GetExperimentalGateCount(0) == [int(x) for x in counts[2:2 + n]]


def test_noisy_qureg_plain_gates_add_no_noise():
    """Gates NoisyQureg does not override run without noise (the reference's are not virtual)."""
    import iqs_gb300 as iqs
    r = iqs.NoisyQureg(3, 11, 5.0, 4.0)
    r.Initialize("base", 0)
    r.ApplyHadamard(0)
    r.ApplyPauliX(1)
    r.ApplyCPauliZ(0, 1)
    r.ApplyCRotationX(1, 2, 0.4)
    assert r.GetTotalExperimentalGateCount() == 1
    ref = iqs.QubitRegister(3, "base", 0)
    ref.ApplyHadamard(0)
    ref.ApplyPauliX(1)
    ref.ApplyCPauliZ(0, 1)
    ref.ApplyCRotationX(1, 2, 0.4)
    assert np.max(np.abs(r.GetStateVector() - ref.GetStateVector())) <= 1e-15


@pytest.mark.parametrize("key", _groups("channel"))
def test_channels_match_reference(key):
    """ApplyChannel (src/qureg_apply_channel.cpp:17-106) with the eigensystems of the fixture:
    the same draws, gates and overall sign."""
    import iqs_gb300 as iqs
    z = np.load(FIX)
    meta = json.loads(str(z[f"{key}/meta"]))
    prec = meta["precision"]
    sysname = f"chinorm/{meta['system']}_{prec.lower()}"
    ev, vecs = z[f"{sysname}/evals"], z[f"{sysname}/evecs"]
    chi = iqs.ChiMatrix(len(ev), precision=prec)
    chi.SetEigenSystem(ev, vecs)
    r = iqs.QubitRegister(meta["n"], "base", 0, precision=prec)
    r.SetStateVector(z[f"{key}/init"])
    rng = iqs.RandomNumberGenerator(precision=prec)
    rng.SetSeedStreamPtrs(meta["seed"])
    r.SetRngPtr(rng)
    qs = meta["qubits"]
    for i in range(meta["steps"]):
        if len(ev) == 4:
            r.ApplyChannel(qs[i], chi)
        else:
            r.ApplyChannel(qs[2 * i], qs[2 * i + 1], chi)
    want = z[f"{key}/state"]
    scale = max(1.0, float(np.max(np.abs(want))))
    assert np.max(np.abs(r.GetStateVector() - want)) <= TOL[prec] * 10 * scale
    assert r.GetOverallSignOfChannels() == float(z[f"{key}/sign"])


@pytest.mark.parametrize("times", [1, 3])
def test_ideal_hadamard_channel(times):
    """ApplyQuantumChannel.IdealHadamard (unit_test/include/qureg_apply_channel.hpp:39-64)."""
    import iqs_gb300 as iqs
    z = np.load(FIX)
    chi = iqs.CM4x4()
    chi[1, 1] = chi[1, 3] = chi[3, 1] = chi[3, 3] = 0.5
    chi.EigensystemOfIdealHadamardChannel()
    psi = iqs.QubitRegister(4, "base", 4)
    rng = iqs.RandomNumberGenerator()
    rng.SetSeedStreamPtrs(7777)
    psi.SetRngPtr(rng)
    psi.ApplyHadamard(2)
    for _ in range(times):
        psi.ApplyChannel(2, chi)
    if times == 1:
        assert abs(psi.GetGlobalAmplitude(4) - 1) <= 1e-15
    assert np.max(np.abs(psi.GetStateVector() - z[f"hadamard/times{times}/state"])) <= 1e-15


def test_depolarizing_channel_average():
    """ApplyQuantumChannel.DepolarizingChannel (qureg_apply_channel.hpp:71-123) with the
    eigensystem from SolveEigenSystem: over many trajectories <X> of |+> decays as (1 - 4p/3)^t."""
    import iqs_gb300 as iqs
    p, steps, traj = 0.1, 4, 400
    chi = iqs.CM4x4()
    for i in range(4):
        chi[i, i] = 1 - p if i == 0 else p / 3
    chi.SolveEigenSystem()
    rng = iqs.RandomNumberGenerator()
    rng.SetSeedStreamPtrs(7777)
    acc = 0.0
    psi = iqs.QubitRegister(2, "base", 0)
    psi.SetRngPtr(rng)
    for _ in range(traj):
        psi.Initialize("base", 0)
        psi.ApplyHadamard(0)
        for _ in range(steps):
            psi.ApplyChannel(0, chi)
        acc += psi.ExpectationValue([0], [1], 1.0) * psi.GetOverallSignOfChannels()
    want = (1 - 4 * p / 3) ** steps
    assert abs(acc / traj - want) < 0.12
    with pytest.raises(ValueError):
        psi.ApplyChannel(0, 1, chi)  # a 4x4 chi on two qubits


@pytest.fixture(scope="module")
def noise_driver(tmp_path_factory):
    import subprocess
    d = tmp_path_factory.mktemp("noise")
    exe = d / "noise_driver"
    libdir = REPO / "intel-qs_gb300" / "iqs_gb300"
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", str(REPO / "include"), str(REPO / "tests" / "cpp" / "noise_driver.cpp"),
                    "-L", str(libdir), "-liqsg", f"-Wl,-rpath,{libdir}", "-o", str(exe)], check=True)
    return exe


def _run(exe, mode, text):
    import subprocess
    r = subprocess.run([str(exe), mode], input=text, capture_output=True, text=True, check=True)
    return [l for l in r.stdout.split("\n") if l]


def _amps(psi):
    return "".join(f"{float(x.real)!r} {float(x.imag)!r}\n" for x in psi)


def _state(lines, n):
    return np.array([complex(*map(float, l.split())) for l in lines[:1 << n]])


@pytest.mark.parametrize("key", ["noise/unit_test_6q_dp", "noise/random_8q_sp"])
def test_cpp_noise_gates_match_reference(noise_driver, key):
    """QubitRegister::ApplyNoiseGate of the C++ drop-in header with iqs::RandomNumberGenerator."""
    z = np.load(FIX)
    meta = json.loads(str(z[f"{key}/meta"]))
    prec, n = meta["precision"], meta["n"]
    text = f"{1 if prec == 'SP' else 0} {n} {meta['seed']} {meta['T1']!r} {meta['T2']!r} {len(meta['qubits'])}\n"
    text += _amps(z[f"{key}/init"]) + "".join(f"{q} {d!r}\n" for q, d in zip(meta["qubits"], meta["durations"]))
    out = _run(noise_driver, "noise", text)
    assert np.max(np.abs(_state(out, n) - z[f"{key}/state"])) <= TOL[prec]
    assert [int(x) for x in out[1 << n].split()[1:]] == [int(x) for x in z[f"{key}/counts"]]


@pytest.mark.parametrize("key", ["noisy/strong_dp", "noisy/defaults_sp"])
def test_cpp_noisy_qureg_matches_reference(noise_driver, key):
    """iqs::NoisyQureg of the C++ drop-in header."""
    z = np.load(FIX)
    meta = json.loads(str(z[f"{key}/meta"]))
    prec, n = meta["precision"], meta["n"]
    text = (f"{1 if prec == 'SP' else 0} {n} {meta['seed']} {meta['T1']!r} {meta['T2']!r} {meta['Ts']!r} "
            f"{meta['Td']!r} {len(meta['prog'])}\n")
    for (kind, a, b), ang, m in zip(meta["prog"], meta["angles"], z[f"{key}/mats"]):
        text += f"{kind} {a} {b} {ang!r} " + " ".join(f"{float(x.real)!r} {float(x.imag)!r}" for x in m) + "\n"
    out = _run(noise_driver, "noisy", text)
    assert np.max(np.abs(_state(out, n) - z[f"{key}/state"])) <= TOL[prec] * 10
    assert [int(x) for x in out[1 << n].split()[1:]] == [int(x) for x in z[f"{key}/counts"]]


@pytest.mark.parametrize("key", ["channel/m4_mixed_dp", "channel/m16_mixed_sp"])
def test_cpp_channels_match_reference(noise_driver, key):
    """QubitRegister::ApplyChannel of the C++ drop-in header with iqs::ChiMatrix."""
    z = np.load(FIX)
    meta = json.loads(str(z[f"{key}/meta"]))
    prec, n = meta["precision"], meta["n"]
    sysname = f"chinorm/{meta['system']}_{prec.lower()}"
    ev, vecs = z[f"{sysname}/evals"], z[f"{sysname}/evecs"]
    text = f"{1 if prec == 'SP' else 0} {n} {meta['seed']} {len(ev)} {meta['steps']}\n"
    text += _amps(ev) + _amps(vecs.reshape(-1)) + _amps(z[f"{key}/init"])
    text += " ".join(map(str, meta["qubits"])) + "\n"
    out = _run(noise_driver, "channel", text)
    want = z[f"{key}/state"]
    scale = max(1.0, float(np.max(np.abs(want))))
    assert np.max(np.abs(_state(out, n) - want)) <= TOL[prec] * 10 * scale
    assert float(out[1 << n].split()[1]) == float(z[f"{key}/sign"])


def test_qubit_register_metric_counts_and_depth():
    """QubitRegisterMetric (include/QubitRegisterMetric.hpp): counts and parallel depth of the
    counted gates; the state equals a plain register's."""
    import iqs_gb300 as iqs
    r = iqs.QubitRegisterMetric(4)
    r.Initialize("base", 0)
    plain = iqs.QubitRegister(4, "base", 0)
    for reg in (r, plain):
        reg.ApplyHadamard(0)
        reg.ApplyRotationX(1, 0.3)
        reg.ApplyCPauliX(0, 1)
        reg.ApplyRotationZ(3, 1.1)
        reg.ApplyControlled1QubitGate(1, 2, np.array([[0, 1], [1, 0]], dtype=complex))
        reg.ApplyPauliY(3)  # not counted
    assert (r.GetOneQubitGateCount(), r.GetTwoQubitGateCount(), r.GetTotalQubitGateCount()) == (3, 2, 5)
    # depths: q0 1 -> 2 (CX with q1 at 1), q1 -> 2 -> 3 (CU with q2 at 0), q2 -> 3, q3 -> 1
    assert r.GetParallelDepth() == 3
    assert np.max(np.abs(r.GetStateVector() - plain.GetStateVector())) <= 1e-15
