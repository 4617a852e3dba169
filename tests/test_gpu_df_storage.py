"""Emulated-ComplexDP gate streams with the state held as double-float pairs between sweeps
(IQSG_OPT_DF_STORAGE): agreement with the oracle and with FP64 storage, the range check that
sends a run back to FP64 storage, the host check on non-contractive gates, tiny amplitudes,
and the public API reading FP64 amplitudes after a run."""
import numpy as np
import pytest

import oracle
from circuits import brick_layer_ops, enc, haar_2x2, haar_4x4, random_state, replay
from conftest import TOL_DP

pytestmark = pytest.mark.gpu


def _layers(n, rng, count=3):
    ops = []
    for _ in range(count):
        ops += brick_layer_ops(n, rng, "ApplyCPauliZ")
    return ops


def _run(n, ops, *, pairs, width=2, init=None, base=5):
    import iqs_gb300 as iqs
    reg = iqs.QubitRegister(n, "base", base, math="emulated")
    if init is not None:
        reg.SetStateVector(init)
    reg.SetSweepWidth(width)
    reg.SetDoubleFloatStorage(pairs)
    reg.TurnOnFusion()
    replay(reg, ops)
    reg.ApplyFusedGates()
    return reg


@pytest.mark.parametrize("width", [1, 2, 3])
def test_pairs_match_oracle_and_fp64_storage(width):
    n = 16
    ops = _layers(n, np.random.default_rng(41))
    a = _run(n, ops, pairs=True, width=width)
    b = _run(n, ops, pairs=False, width=width)
    assert a.counters()["df_runs"] == 1 and b.counters()["df_runs"] == 0
    ref = oracle.OracleRegister(n, "base", 5)
    replay(ref, ops)
    want = ref.GetStateVector()
    assert np.max(np.abs(a.GetStateVector() - want)) <= TOL_DP
    assert np.max(np.abs(a.GetStateVector() - b.GetStateVector())) <= 1e-14
    assert abs(a.GetProbability(3) - ref.GetProbability(3)) <= TOL_DP
    assert abs(a.ComputeNorm() - 1.0) <= 1e-13


def test_two_qubit_gates_and_runs_in_a_row():
    import iqs_gb300 as iqs
    n = 14
    rng = np.random.default_rng(42)
    reg = iqs.QubitRegister(n, "base", 0, math="emulated")
    ref = oracle.OracleRegister(n, "base", 0)
    reg.TurnOnFusion()
    for _ in range(3):
        ops = [["Apply1QubitGate", [q, enc(haar_2x2(rng))]] for q in range(n)]
        ops += [["Apply2QubitGate", [q + 1, q, enc(haar_4x4(rng))]] for q in range(0, n - 1, 2)]
        ops.append(["ApplyCPauliX", [2, 9]])
        replay(reg, ops)
        replay(ref, ops)
        reg.ApplyFusedGates()
    assert reg.counters()["df_runs"] == 3
    assert np.max(np.abs(reg.GetStateVector() - ref.GetStateVector())) <= TOL_DP


def test_out_of_range_state_takes_fp64_storage():
    """A component of 2^80 fails the range check on the device: every sweep runs the FP64
    storage kernel instead, with the same result bit for bit."""
    n = 12
    rng = np.random.default_rng(43)
    init = random_state(n, rng)
    init[17] = 2.0 ** 80
    ops = _layers(n, rng)
    a = _run(n, ops, pairs=True, init=init)
    b = _run(n, ops, pairs=False, init=init)
    assert a.counters()["df_runs"] == 1
    assert np.array_equal(a.GetStateVector(), b.GetStateVector())


def test_non_contractive_gate_stays_on_fp64_storage():
    import iqs_gb300 as iqs
    n = 12
    rng = np.random.default_rng(44)
    ops = _layers(n, rng)
    ops.append(["Apply1QubitGate", [4, enc(1.5 * haar_2x2(rng))]])
    regs = []
    for pairs in (True, False):
        reg = iqs.QubitRegister(n, "base", 3, math="emulated")
        reg.SetDoubleFloatStorage(pairs)
        reg.TurnOnFusion()
        replay(reg, ops)
        reg.ApplyFusedGates()
        regs.append(reg)
    assert regs[0].counters()["df_runs"] == 0
    assert np.array_equal(regs[0].GetStateVector(), regs[1].GetStateVector())


def test_tiny_amplitudes_keep_relative_accuracy():
    """A state scaled by 1e-30 (below the split's fast range) runs as pairs; its amplitudes keep
    their relative accuracy."""
    n = 12
    rng = np.random.default_rng(45)
    init = random_state(n, rng) * 1e-30
    ops = _layers(n, rng)
    a = _run(n, ops, pairs=True, init=init)
    assert a.counters()["df_runs"] == 1
    ref = oracle.OracleRegister(n, "base", 0)
    ref.SetStateVector(init)
    replay(ref, ops)
    want = ref.GetStateVector()
    assert np.max(np.abs(a.GetStateVector() - want)) <= TOL_DP * 1e-30


def test_short_streams_keep_fp64_storage():
    n = 12
    ops = brick_layer_ops(n, np.random.default_rng(46), "ApplyCPauliZ")[:3]
    a = _run(n, ops, pairs=True, width=2)
    assert a.counters()["df_runs"] == 0
