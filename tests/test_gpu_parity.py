"""Parity of the GPU engine (libiqsg through iqs_gb300.QubitRegister) with the reference:
golden vectors the reference produced, and the pinned C oracle on larger seeded circuits.
Bars: per-amplitude max abs error <= 1e-12 (ComplexDP) and <= 2e-5 (ComplexSP); qubit maps
and permuted index placement bit-exact."""
import math

import numpy as np
import pytest

import oracle
from circuits import brick_layer_ops, enc, haar_2x2, random_circuit, random_state, replay
from conftest import TOL_DP, TOL_SP, case_meta, case_ops, compare_final, golden_cases

pytestmark = pytest.mark.gpu

MODES = [("DP", "native"), ("DP", "emulated"), ("SP", "native")]


@pytest.fixture(scope="module")
def iqs():
    import iqs_gb300
    return iqs_gb300


def _gpu_reg(iqs, n, prec, math_mode, style="base", base=0):
    return iqs.QubitRegister(n, style, base, precision=prec, math=math_mode)


@pytest.mark.parametrize("fused", [False, True])
@pytest.mark.parametrize("math_mode", ["native", "emulated"])
@pytest.mark.parametrize("prefix", ["kat_", "random_", "collapse_", "fusion_", "plain_"])
def test_golden_cases(iqs, golden, prefix, math_mode, fused):
    for name in golden_cases(golden, prefix):
        meta = case_meta(golden, name)
        prec = meta["precision"]
        reg = _gpu_reg(iqs, meta["n"], prec, math_mode, meta["style"], meta["base"])
        if f"{name}/init" in golden:
            reg.SetStateVector(golden[f"{name}/init"])
        if fused or meta.get("fusion") is not None:
            reg.TurnOnFusion(meta.get("fusion") or 20)
        q = np.asarray(replay(reg, case_ops(golden, name)))
        if fused or meta.get("fusion") is not None:
            reg.TurnOffFusion()
        tol = TOL_DP if prec == "DP" else TOL_SP
        err = compare_final(golden, name, reg.GetStateVector().astype(np.complex128), tol)
        assert err <= tol, f"{name} ({math_mode}): max abs error {err:.3e} > {tol}"
        assert reg.qubit_permutation.map == [int(x) for x in golden[f"{name}/map"]], f"{name}: map differs"
        gq = golden[f"{name}/queries"]
        if gq.size:
            qerr = float(np.max(np.abs(q - gq)))
            assert qerr <= tol, f"{name} ({math_mode}): query error {qerr:.3e}"


@pytest.mark.parametrize("name", ["qaoa_ring6", "qaoa_random10"])
def test_golden_qaoa(iqs, golden, name):
    import json
    meta = json.loads(str(golden[f"{name}/meta"]))
    n = meta["n"]
    diag = iqs.QubitRegister(n, "base", 0)
    mx = iqs.InitializeVectorAsMaxCutCostFunction(diag, golden[f"{name}/adjacency"])
    assert mx == int(golden[f"{name}/max_cut"])
    assert np.array_equal(diag.GetStateVector().real, golden[f"{name}/cost"])
    psi = iqs.QubitRegister(n, "++++", 0)
    for g, b in zip(meta["gammas"], meta["betas"]):
        iqs.ImplementQaoaLayerBasedOnCostFunction(psi, diag, g)
        for q in range(n):
            psi.ApplyRotationX(q, 2 * b)
    assert np.max(np.abs(psi.GetStateVector() - golden[f"{name}/final"])) <= TOL_DP
    e1 = iqs.GetExpectationValueFromCostFunction(psi, diag)
    e2 = iqs.GetExpectationValueSquaredFromCostFunction(psi, diag)
    assert np.allclose([e1, e2], golden[f"{name}/expectation"], rtol=0, atol=1e-11)


@pytest.mark.parametrize("prec,math_mode", MODES)
@pytest.mark.parametrize("n,seed", [(14, 201), (17, 202)])
def test_random_circuits_vs_oracle(iqs, n, seed, prec, math_mode):
    rng = np.random.default_rng(seed)
    init = random_state(n, rng)
    ops = random_circuit(n, 250, rng)
    a = oracle.OracleRegister(n, "base", 0, prec)
    a.SetStateVector(init)
    b = _gpu_reg(iqs, n, prec, math_mode)
    b.SetStateVector(init)
    qa, qb = np.asarray(replay(a, ops)), np.asarray(replay(b, ops))
    tol = TOL_DP if prec == "DP" else TOL_SP
    assert np.max(np.abs(a.GetStateVector() - b.GetStateVector())) <= tol
    assert a.perm.map == b.qubit_permutation.map
    assert np.max(np.abs(qa - qb), initial=0.0) <= tol


@pytest.mark.parametrize("prec,math_mode", MODES)
@pytest.mark.parametrize("width", [1, 2, 3, 4])
@pytest.mark.parametrize("n,seed,nops,pipeline", [(6, 601, 300, False), (13, 602, 300, False),
                                                  (18, 603, 120, False), (18, 604, 120, True)])
def test_fused_sweeps_vs_oracle(iqs, n, seed, nops, pipeline, width, prec, math_mode):
    """Fused sweeps of every width over mixed circuits (1q, controlled, 2q dense, swap family,
    diagonal, Toffoli) against the oracle applying the same gates one by one, with the direct
    and (from 16 qubits) the bulk-copy pipelined kernels."""
    rng = np.random.default_rng(seed)
    init = random_state(n, rng)
    ops = random_circuit(n, nops, rng, permutes=True, queries=True)
    a = oracle.OracleRegister(n, "base", 0, prec)
    a.SetStateVector(init)
    b = _gpu_reg(iqs, n, prec, math_mode)
    b.SetStateVector(init)
    b.SetSweepWidth(width)
    b.SetSweepPipeline(pipeline)
    b.TurnOnFusion()
    qa, qb = np.asarray(replay(a, ops)), np.asarray(replay(b, ops))
    b.TurnOffFusion()
    tol = TOL_DP if prec == "DP" else TOL_SP
    assert np.max(np.abs(a.GetStateVector() - b.GetStateVector())) <= tol
    assert np.max(np.abs(qa - qb), initial=0.0) <= tol


def test_fused_native_is_bit_identical_to_unfused(iqs):
    """In native FP64 a fused sweep performs the same operations as the per-gate kernels."""
    n = 12
    rng = np.random.default_rng(701)
    init = random_state(n, rng)
    ops = brick_layer_ops(n, rng, "ApplyCPauliZ") + brick_layer_ops(n, rng, "ApplyCPauliX")
    a = iqs.QubitRegister(n, "base", 0)
    b = iqs.QubitRegister(n, "base", 0)
    a.SetStateVector(init)
    b.SetStateVector(init)
    replay(a, ops)
    b.TurnOnFusion()
    replay(b, ops)
    sweeps = b.ApplyFusedGates()
    assert 0 < sweeps < len(ops)
    assert np.array_equal(a.GetStateVector(), b.GetStateVector())


@pytest.mark.parametrize("prec,math_mode", MODES)
def test_every_position_and_pair(iqs, prec, math_mode):
    """Every target position of a 1-qubit gate and every (control, target) pair (the
    low-position shuffle and high-position strided cases alike)."""
    n = 9
    rng = np.random.default_rng(301)
    init = random_state(n, rng)
    ops = [["Apply1QubitGate", [q, enc(haar_2x2(rng))]] for q in range(n)]
    ops += [["ApplyControlled1QubitGate", [c, t, enc(haar_2x2(rng))]] for c in range(n) for t in range(n) if c != t]
    ops += [["ApplySwap", [a, b]] for a in range(n) for b in range(a + 1, n)]
    ops += [["ApplyToffoli", [a, b, c]] for a, b, c in ((0, 1, 2), (8, 0, 4), (3, 7, 1), (5, 2, 8))]
    a = oracle.OracleRegister(n, "base", 0, prec)
    a.SetStateVector(init)
    b = _gpu_reg(iqs, n, prec, math_mode)
    b.SetStateVector(init)
    replay(a, ops)
    replay(b, ops)
    tol = TOL_DP if prec == "DP" else TOL_SP
    assert np.max(np.abs(a.GetStateVector() - b.GetStateVector())) <= tol


@pytest.mark.parametrize("prec", ["DP", "SP"])
def test_permutation_bit_exact(iqs, prec):
    """Amplitude k holds the integer k: after any reorder every value must sit exactly where
    the oracle puts it (index placement is integer work: no tolerance)."""
    n = 16
    rng = np.random.default_rng(401)
    vals = np.arange(1 << n, dtype=np.float64) + 1j * (np.arange(1 << n) % 7)
    a = oracle.OracleRegister(n, "base", 0, prec)
    b = iqs.QubitRegister(n, "base", 0, precision=prec)
    a.SetStateVector(vals)
    b.SetStateVector(vals)
    for _ in range(5):
        m = [int(x) for x in rng.permutation(n)]
        style = "direct" if rng.random() < 0.5 else "inverse"
        a.PermuteQubits(m, style)
        b.PermuteQubits(m, style)
        assert np.array_equal(a.GetStateVector(), b.GetStateVector())
        assert a.perm.map == b.qubit_permutation.map
    # GetGlobalAmplitude addresses program qubits through the map.
    for idx in rng.integers(0, 1 << n, size=50):
        assert b.GetGlobalAmplitude(int(idx)) == a.GetGlobalAmplitude(int(idx))


def test_swap_equals_three_cnots_exactly(iqs):
    """unit_test/include/apply_swap_gate_test.hpp:111: SWAP and CNOT^3 agree exactly."""
    n = 12
    rng = np.random.default_rng(7777)
    init = random_state(n, rng)
    for q1, q2 in ((0, 1), (3, 11), (10, 2)):
        a = iqs.QubitRegister(n, "base", 0)
        b = iqs.QubitRegister(n, "base", 0)
        a.SetStateVector(init)
        b.SetStateVector(init)
        a.ApplySwap(q1, q2)
        b.ApplyCPauliX(q1, q2)
        b.ApplyCPauliX(q2, q1)
        b.ApplyCPauliX(q1, q2)
        assert a.MaxAbsDiff(b) == 0.0


def test_plain_gate_by_gate_20q_expectations(iqs, golden):
    """The 20-qubit, 780-gate circuit: <Z0 Z19> and the norm against the reference."""
    name = "plain_gate_by_gate_20q"
    for math_mode in ("native", "emulated"):
        reg = iqs.QubitRegister(20, "base", 0, math=math_mode)
        q = replay(reg, case_ops(golden, name))
        assert np.max(np.abs(np.asarray(q) - golden[f"{name}/queries"])) <= TOL_DP


def test_invalid_arguments_raise(iqs):
    r = iqs.QubitRegister(5, "base", 0)
    with pytest.raises(ValueError):
        r.ApplyHadamard(5)
    with pytest.raises(ValueError):
        r.ApplyCPauliX(2, 2)
    with pytest.raises(ValueError):
        r.Apply1QubitGate(0, np.eye(3))
    with pytest.raises(ValueError):
        r.PermuteQubits([0, 1, 2, 3, 3])
    with pytest.raises(ValueError):
        r.ExpectationValue([0, 0], [3, 3])
    with pytest.raises(ValueError):
        r.ExpectationValue([0], [4])
    with pytest.raises(ValueError):
        r.ApplyToffoli(1, 1, 2)
    other = iqs.QubitRegister(4, "base", 0)
    with pytest.raises(ValueError):
        r.ComputeOverlap(other)
    # the register is still usable afterwards
    r.ApplyHadamard(0)
    assert abs(r.GetProbability(0) - 0.5) < 1e-15


def test_allocation_failure_is_reported(iqs):
    """A 40-qubit ComplexDP register (16 TiB) cannot be allocated: MemoryError, and the
    device stays usable (host-side fault injection; nothing faults on the GPU)."""
    with pytest.raises(MemoryError):
        iqs.QubitRegister(40, "base", 0)
    r = iqs.QubitRegister(3, "base", 0)
    r.ApplyPauliX(2)
    assert r.GetProbability(2) == 1.0


def test_wrapped_device_memory_and_cuda_array_interface(iqs):
    torch = pytest.importorskip("torch")
    n = 10
    t = torch.zeros(1 << n, dtype=torch.complex128, device="cuda")
    t[3] = 1.0
    torch.cuda.synchronize()
    r = iqs.QubitRegister.from_device(n, t.data_ptr())
    r.ApplyHadamard(0)
    r.synchronize()
    v = t.cpu().numpy()
    assert abs(v[2] - 1 / math.sqrt(2)) < 1e-15 and abs(v[3] + 1 / math.sqrt(2)) < 1e-15
    view = torch.as_tensor(r, device="cuda")
    assert view.data_ptr() == t.data_ptr()


@pytest.mark.parametrize("math_mode", ["native", "emulated"])
def test_large_register_properties(iqs, math_mode):
    """26 qubits (1 GiB): a layer of Haar gates and CZ bricks preserves the norm, and
    applying the inverse layer restores the initial state."""
    n = 26
    rng = np.random.default_rng(501)
    ops = brick_layer_ops(n, rng, "ApplyCPauliZ")
    r = iqs.QubitRegister(n, "base", 0, math=math_mode)
    for q in range(n):
        r.ApplyHadamard(q)
    r.ApplyRotationZ(3, 0.3)
    ref = iqs.QubitRegister(r)
    replay(r, ops)
    assert abs(r.ComputeNorm() - 1.0) < 1e-12
    inv = []
    for name, args in reversed(ops):
        if name == "Apply1QubitGate":
            m = np.array([[complex(*x) for x in row] for row in args[1]])
            inv.append(["Apply1QubitGate", [args[0], enc(m.conj().T)]])
        else:
            inv.append([name, args])
    replay(r, inv)
    assert r.MaxAbsDiff(ref) <= 1e-12
