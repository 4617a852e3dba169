"""Shared-memory tile passes (IQSG_OPT_TILE_QUBITS): gate streams run as tile passes agree
with the oracle and with register sweeps, in ComplexDP (native arithmetic) and ComplexSP;
adjoint tile passes give the same gradients as adjoint register sweeps; a stream too long
for one pass's parameter block is split."""
import math

import numpy as np
import pytest

import oracle
from circuits import random_circuit, replay
from conftest import TOL_DP, TOL_SP

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision,tol", [("DP", TOL_DP), ("SP", TOL_SP)])
@pytest.mark.parametrize("tile", [8, 11, 13])
def test_random_circuits_in_tiles(precision, tol, tile):
    import iqs_gb300 as iqs
    n = 16
    rng = np.random.default_rng(100 + tile)
    ops = random_circuit(n, 400, rng, permutes=False, queries=False)
    init = rng.standard_normal(1 << n) + 1j * rng.standard_normal(1 << n)
    init /= np.linalg.norm(init)
    reg = iqs.QubitRegister(n, "", 0, precision=precision)
    reg.SetStateVector(init)
    reg.SetTileQubits(tile)
    reg.TurnOnFusion()
    replay(reg, ops)
    passes = reg.ApplyFusedGates()
    ref = oracle.OracleRegister(n, "", 0, precision)
    ref.SetStateVector(init)
    replay(ref, ops)
    assert np.max(np.abs(reg.GetStateVector() - ref.GetStateVector())) <= tol
    assert 0 < passes < len(ops)


def test_tile_passes_fewer_than_register_sweeps():
    import iqs_gb300 as iqs
    n = 20
    rng = np.random.default_rng(5)
    ops = []
    for _ in range(6):
        for q in range(n):
            z = rng.standard_normal((2, 2)) + 1j * rng.standard_normal((2, 2))
            ops.append(["Apply1QubitGate", [q, np.linalg.qr(z)[0]]])
        for q in range(0, n - 1, 2):
            ops.append(["ApplyCPauliX", [q, q + 1]])
    counts = {}
    states = {}
    for tile in (0, 12):
        reg = iqs.QubitRegister(n, "base", 0, precision="SP")
        reg.SetTileQubits(tile)
        reg.TurnOnFusion()
        for name, args in ops:
            getattr(reg, name)(*args)
        counts[tile] = reg.ApplyFusedGates()
        states[tile] = reg.GetStateVector()
    assert counts[12] * 2 < counts[0]
    assert np.max(np.abs(states[12] - states[0])) <= 1e-5


def test_long_stream_splits_parameter_block():
    """Hundreds of gates inside one tile's positions: the pass is split, results unchanged."""
    import iqs_gb300 as iqs
    n = 14
    rng = np.random.default_rng(9)
    ops = []
    for k in range(600):
        q = int(rng.integers(0, 6))
        ops.append(["ApplyRotationY", [q, float(rng.uniform(-3, 3))]])
        ops.append(["ApplyCPhaseRotation", [q, int(rng.integers(6, n)), float(rng.uniform(-3, 3))]])
    reg = iqs.QubitRegister(n, "base", 3)
    reg.SetTileQubits(10)
    reg.TurnOnFusion()
    replay(reg, ops)
    passes = reg.ApplyFusedGates()
    ref = oracle.OracleRegister(n, "base", 3)
    replay(ref, ops)
    assert passes >= 2
    assert np.max(np.abs(reg.GetStateVector() - ref.GetStateVector())) <= TOL_DP


@pytest.mark.parametrize("precision", ["DP", "SP"])
def test_trotter_in_tiles(precision):
    from iqs_gb300.trotter import XXZChain, bond_gate, strang_layers
    n, steps = 16, 6
    J = np.random.default_rng(4).uniform(0.5, 1.5, n - 1)
    o = oracle.OracleRegister(n, "base", sum(1 << q for q in range(1, n, 2)))
    for bonds, tau in strang_layers(n, 0.05, steps):
        for b in bonds:
            o.Apply2QubitGate(b + 1, b, bond_gate(0.5 * tau * J[b], 0.8))
    tol = TOL_DP if precision == "DP" else TOL_SP
    plain = XXZChain(n, J, steps=steps, precision=precision, checkpoint_every=3)
    e0, g0 = plain.energy_and_grad()
    tiled = XXZChain(n, J, steps=steps, precision=precision, checkpoint_every=3, tile_qubits=11)
    zz = tiled.bond_zz()
    assert np.max(np.abs(tiled.psi.GetStateVector() - o.GetStateVector())) <= tol
    assert tiled.sweeps_forward * 2 < plain.sweeps_forward or plain.sweeps_forward == 0
    e1, g1 = tiled.energy_and_grad()
    assert abs(e1 - e0) <= (1e-12 if precision == "DP" else 1e-5)
    assert np.max(np.abs(g1 - g0)) <= (1e-11 if precision == "DP" else 1e-4) * max(1.0, np.max(np.abs(g0)))
    assert tiled.sweeps_backward < plain.sweeps_backward
    assert len(zz) == n - 1
