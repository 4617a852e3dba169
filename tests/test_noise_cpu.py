"""Host side of the noise paths, without a GPU: the random number streams and the chi-matrix
normalisation against the reference's own outputs (tests/golden/noise.npz, made by
tests/golden/make_noise.py), the noise-gate matrix against its closed form, and the chi-matrix
eigensystem against the channel it must reproduce on average."""
import ctypes as C
import json

import numpy as np
import pytest

from conftest import REPO

FIX = REPO / "tests" / "golden" / "noise.npz"
PAULI = [np.eye(2), np.array([[0, 1], [1, 0]]), np.array([[0, -1j], [1j, 0]]), np.array([[1, 0], [0, -1]])]


def _groups(prefix):
    z = np.load(FIX)
    return sorted({"/".join(k.split("/")[:2]) for k in z.files if k.startswith(prefix + "/")})


def _dp(a):
    from iqs_gb300 import _lib
    return a.ctypes.data_as(_lib._DP)


@pytest.mark.parametrize("key", _groups("rng"))
def test_random_streams_match_reference(key):
    """Uniforms, Gaussians, integers, skips and the copy constructor of RandomNumberGenerator
    (src/rng_utils.cpp:13-225): the same values and the same counts."""
    import iqs_gb300 as iqs
    z = np.load(FIX)
    meta = json.loads(str(z[f"{key}/meta"]))
    rng = iqs.RandomNumberGenerator(precision=meta["precision"])
    rng.SetSeedStreamPtrs(meta["seed"])
    names = ["pool", "state", "local"]
    got = []
    for kind, n, st in meta["ops"]:
        s = names[st]
        if kind == 0:
            got += list(rng.UniformRandomNumbers(n, 0, 1, s))
        elif kind == 1:
            got += list(rng.UniformRandomNumbers(n, -2, 5, s))
        elif kind == 2:
            got += list(rng.GaussianRandomNumbers(n, s))
        elif kind == 3:
            got += list(rng.RandomIntegersInRange(n, -3, 17, s))
        elif kind == 4:
            rng.SkipAhead(n, s)
        elif kind == 5:
            rng = iqs.RandomNumberGenerator(rng)
    want = z[f"{key}/values"]
    assert np.array_equal(np.array(got, dtype=np.float64), want)
    counts = [rng.GetNumGeneratedOrSkippedPoolNumbers(), rng.GetNumGeneratedOrSkippedStateNumbers(),
              rng.GetNumGeneratedOrSkippedLocalNumbers()]
    assert counts == [int(x) for x in z[f"{key}/counts"]]


def test_random_streams_reference_unit_tests():
    """RandomNumberGeneratorTest.BasicUse / DifferentSeed / SkipMethod
    (unit_test/include/random_number_generator_test.hpp:36-178)."""
    import iqs_gb300 as iqs
    a, b = iqs.RandomNumberGenerator(), iqs.RandomNumberGenerator()
    a.SetSeedStreamPtrs(777)
    b.SetSeedStreamPtrs(777)
    x, y = a.UniformRandomNumbers(10, 0, 1, "local"), b.UniformRandomNumbers(10, 0.0, 1.0)
    assert x[0] != x[-1] and np.array_equal(x, y)
    assert (a.GetNumGeneratedOrSkippedLocalNumbers(), a.GetNumGeneratedOrSkippedStateNumbers(),
            a.GetNumGeneratedOrSkippedPoolNumbers()) == (10, 0, 0)
    c, d = iqs.RandomNumberGenerator(), iqs.RandomNumberGenerator()
    c.SetSeedStreamPtrs(717)
    d.SetSeedStreamPtrs(718)
    assert not set(c.UniformRandomNumbers(100)) & set(d.UniformRandomNumbers(100))
    e, f = iqs.RandomNumberGenerator(), iqs.RandomNumberGenerator()
    e.SetSeedStreamPtrs(717)
    f.SetSeedStreamPtrs(717)
    full = e.UniformRandomNumbers(80, 0, 1, "local")
    f.SkipAhead(40, "local")
    assert np.array_equal(full[40:], f.UniformRandomNumbers(40, 0, 1, "local"))
    assert e.GetNumGeneratedOrSkippedLocalNumbers() == f.GetNumGeneratedOrSkippedLocalNumbers()
    g_full = e.GaussianRandomNumbers(80, "local")
    f.GaussianRandomNumbers(40, "local")
    assert np.array_equal(g_full[40:], f.GaussianRandomNumbers(40, "local"))
    with pytest.raises(ValueError):
        e.SkipAhead(3, "global")


@pytest.mark.parametrize("key", _groups("chinorm"))
def test_chi_normalisation_matches_reference(key):
    """NormalizeEigenProbAndRenormalizeEigenVect (src/chi_matrix.cpp:166-200) in the base type."""
    import iqs_gb300 as iqs
    z = np.load(FIX)
    prec = key.rsplit("_", 1)[1].upper()
    ev, vecs = z[f"{key}/evals"], z[f"{key}/evecs"]
    chi = iqs.ChiMatrix(len(ev), precision=prec)
    chi.SetEigenSystem(ev, vecs)
    assert np.array_equal(np.array(chi.GetEigenProbabilities()), z[f"{key}/probs"])
    assert np.array_equal(np.array(chi.GetEigenCumulativeProbabilities()), z[f"{key}/cumprobs"])
    assert np.array_equal(np.array(chi.GetEigenVectors(), dtype=np.complex128), z[f"{key}/vecs"])


def test_chi_eigensystem_reference_unit_test():
    """chimatrix_testeigen (unit_test/include/chi_matrix_test.hpp:136-172): eigenvalues of
    [[1, 3], [3, 7]] and the normalised eigenvectors, the latter up to a phase."""
    import iqs_gb300 as iqs
    chi = iqs.ChiMatrix(2, [[1, 3], [3, 7]])
    chi.SolveEigenSystem()
    assert abs(chi.GetEigenValue(0) - -0.24264069) < 1e-7
    assert abs(chi.GetEigenValue(1) - 8.24264069) < 1e-7
    for k, want in ((0, [-2.69121547, 1.11473795]), (1, [-1.11473795, -2.69121547])):
        v = np.array(chi.GetEigenVector(k))
        phase = v[0] / want[0]
        assert abs(abs(phase) - 1) < 1e-7
        assert np.max(np.abs(v - phase * np.array(want))) < 1e-7


def _channel(chi, rho, two):
    paulis = PAULI if not two else [np.kron(a, b) for a in PAULI for b in PAULI]
    out = np.zeros_like(rho)
    for i, si in enumerate(paulis):
        for j, sj in enumerate(paulis):
            out += chi[i, j] * si @ rho @ sj.conj().T
    return out


def _forced_gate(chi, k, seed=11):
    """The gate ApplyChannel builds from eigenvector k (cumulative probabilities set so that any
    draw selects k)."""
    import iqs_gb300 as iqs
    from iqs_gb300._lib import check, lib
    M = chi.M
    ev, _, vf = chi._arrays()
    cum = np.where(np.arange(M) >= k, 1.0, 0.0)
    rng = iqs.RandomNumberGenerator()
    rng.SetSeedStreamPtrs(seed)
    gate = np.zeros(2 * (2 if M == 4 else 4) ** 2)
    kk, neg = C.c_uint(), C.c_int()
    check(lib.iqsg_channel_gate(rng.handle, chi._p, M, _dp(ev), _dp(cum), _dp(vf), _dp(gate), C.byref(kk),
                                C.byref(neg)))
    assert kk.value == k
    d = 2 if M == 4 else 4
    return gate.view(np.complex128).reshape(d, d), -1.0 if neg.value else 1.0


def _check_average(chi_np, two, seed):
    import iqs_gb300 as iqs
    M = chi_np.shape[0]
    chi = iqs.ChiMatrix(M, chi_np)
    chi.SolveEigenSystem()
    rng = np.random.default_rng(seed)
    d = 4 if two else 2
    a = rng.standard_normal((d, d)) + 1j * rng.standard_normal((d, d))
    rho = a @ a.conj().T
    rho /= np.trace(rho)
    avg = np.zeros_like(rho)
    for k in range(M):
        p = chi.GetEigenProbability(k)
        if p == 0:
            continue
        u, sign = _forced_gate(chi, k)
        avg += p * sign * (u @ rho @ u.conj().T)
    assert np.max(np.abs(avg - _channel(chi_np, rho, two))) < 1e-12


def test_channel_average_equals_chi_action_one_qubit():
    """Sum_k p_k sign_k U_k rho U_k^+ = sum_ij chi_ij s_i rho s_j^+ for the eigensystem that
    SolveEigenSystem returns: depolarizing, amplitude damping, and a random complex Hermitian chi
    with negative eigenvalues."""
    p = 0.01
    _check_average(np.diag([1 - p, p / 3, p / 3, p / 3]).astype(complex), False, 1)
    g = 0.3  # amplitude damping: chi_ij = sum_m c_mi conj(c_mj), K_m = sum_i c_mi s_i
    kraus = [np.array([[1, 0], [0, np.sqrt(1 - g)]]), np.array([[0, np.sqrt(g)], [0, 0]])]
    c = np.array([[np.trace(P.conj().T @ K) / 2 for P in PAULI] for K in kraus])
    _check_average(c.T @ c.conj(), False, 2)
    rng = np.random.default_rng(9)
    a = rng.standard_normal((4, 4)) + 1j * rng.standard_normal((4, 4))
    h = (a + a.conj().T) / 8
    _check_average(h, False, 3)


def test_channel_average_equals_chi_action_two_qubits():
    """The same for 16x16 chi matrices with real entries (the 4x4 gate takes its lower triangle as
    the conjugate of the upper one, exact for real eigenvectors): two-qubit depolarizing and a
    random real symmetric chi with negative eigenvalues."""
    p = 0.05
    _check_average(np.diag([1 - p] + [p / 15] * 15).astype(complex), True, 4)
    rng = np.random.default_rng(10)
    a = rng.standard_normal((16, 16))
    _check_average(((a + a.T) / 16).astype(complex), True, 5)


def test_noise_gate_matrix_closed_form():
    """The noise gate is exp(-i vX X) exp(-i vY Y) exp(-i vZ Z) with v = g s / 2,
    s = sqrt(-log(1 - p)) (src/qureg_noisysimul.cpp:33-85)."""
    from iqs_gb300 import _lib
    from iqs_gb300._lib import check, lib
    T1, T2, d = 6.0, 4.0, 1.7
    g = np.array([0.3, -1.2, 0.8])
    m = np.zeros(8)
    check(lib.iqsg_noise_gate_matrix(_lib.COMPLEX_DP, T1, T2, d, _dp(g), _dp(m)))
    u = m.view(np.complex128).reshape(2, 2)
    pX = (1 - np.exp(-d / T1)) / 4
    pZ = (1 - np.exp(-d / T2)) / 2 + (1 - np.exp(-d / T1)) / 4
    v = g * np.sqrt(-np.log(1 - np.array([pX, pX, pZ]))) / 2

    def rot(a, s):
        return np.cos(a) * np.eye(2) - 1j * np.sin(a) * s
    want = rot(v[0], PAULI[1]) @ rot(v[1], PAULI[2]) @ rot(v[2], PAULI[3])
    assert np.max(np.abs(u - want)) < 1e-15
    with pytest.raises(ValueError):  # zero probabilities: the reference asserts p > 0
        check(lib.iqsg_noise_gate_matrix(_lib.COMPLEX_DP, T1, T2, 0.0, _dp(g), _dp(m)))


def test_chi_matrix_checks_and_print(capsys):
    import iqs_gb300 as iqs
    chi = iqs.CM4x4()
    chi[0, 1] = 1.0  # not Hermitian
    with pytest.raises(ValueError):
        chi.SolveEigenSystem()
    with pytest.raises(ValueError):
        chi.EigensystemOfIdealHadamardChannel()
    with pytest.raises(ValueError):
        chi.GetEigenValue(0)
    h = iqs.CM4x4()
    h[1, 1] = h[1, 3] = h[3, 1] = h[3, 3] = 0.5
    h.EigensystemOfIdealHadamardChannel()
    assert h.GetEigenProbabilities() == [1.0, 0.0, 0.0, 0.0]
    s = h.Print(True)
    assert s.startswith("chi_matrix :\n(0,0)\t(0,0)\t(0,0)\t(0,0)\t\n(0,0)\t(0.5,0)\t")
    assert "eigenvector 0 :\n(0,0)\t(0.707107,0)\t(0,0)\t(0.707107,0)\t" in s
    assert capsys.readouterr().out == s


@pytest.fixture(scope="module")
def noise_driver(tmp_path_factory):
    import subprocess
    import iqs_gb300  # noqa: F401  (builds nothing; the library must exist)
    d = tmp_path_factory.mktemp("noise")
    exe = d / "noise_driver"
    libdir = REPO / "intel-qs_gb300" / "iqs_gb300"
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", str(REPO / "include"), str(REPO / "tests" / "cpp" / "noise_driver.cpp"),
                    "-L", str(libdir), "-liqsg", f"-Wl,-rpath,{libdir}", "-o", str(exe)], check=True)
    return exe


def run_driver(exe, mode, text=""):
    import subprocess
    r = subprocess.run([str(exe), mode], input=text, capture_output=True, text=True, check=True)
    return r.stdout.split("\n")


@pytest.mark.parametrize("key", _groups("rng"))
def test_cpp_random_streams_match_reference(noise_driver, key):
    """iqs::RandomNumberGenerator<float|double> of the C++ drop-in header, same sequences."""
    z = np.load(FIX)
    meta = json.loads(str(z[f"{key}/meta"]))
    text = f"{1 if meta['precision'] == 'SP' else 0} {meta['seed']} {len(meta['ops'])}\n"
    text += "".join(f"{k} {n} {s}\n" for k, n, s in meta["ops"])
    out = [l for l in run_driver(noise_driver, "rng", text) if l]
    assert np.array_equal(np.array([float(x) for x in out[:-1]]), z[f"{key}/values"])
    assert [int(x) for x in out[-1].split()[1:]] == [int(x) for x in z[f"{key}/counts"]]


def test_cpp_chi_eigensystem(noise_driver):
    """iqs::ChiMatrix<ComplexDP, 2>::SolveEigenSystem on the reference unit test's matrix."""
    rows = [[float(x) for x in l.split()] for l in run_driver(noise_driver, "eigen") if l]
    assert abs(rows[0][0] - -0.24264069) < 1e-7 and abs(rows[1][0] - 8.24264069) < 1e-7
    for row, want in zip(rows, ([-2.69121547, 1.11473795], [-1.11473795, -2.69121547])):
        v = np.array([complex(row[1], row[2]), complex(row[3], row[4])])
        phase = v[0] / want[0]
        assert abs(abs(phase) - 1) < 1e-7 and np.max(np.abs(v - phase * np.array(want))) < 1e-7
