"""Edge cases of the gate-stream, adjoint, Trotter and batched entry points: empty streams,
one- and two-qubit registers, tile sizes larger than the register, single-qubit batch
instances, adjoint calls without parameters, and rejected inputs."""
import ctypes as C
import math

import numpy as np
import pytest

import oracle
from conftest import TOL_DP

pytestmark = pytest.mark.gpu


def _op(kind, t0, t1=0, m=None, value=0):
    from iqs_gb300 import _lib
    op = _lib.Op()
    op.kind, op.t0, op.t1, op.value = kind, t0, t1, value
    if m is not None:
        a = np.ascontiguousarray(m, dtype=np.complex128).reshape(-1).view(np.float64)
        C.memmove(op.m, a.ctypes.data, a.nbytes)
    return op


def test_empty_stream_and_empty_adjoint():
    import iqs_gb300 as iqs
    from iqs_gb300._lib import check, lib
    a = iqs.QubitRegister(5, "base", 3)
    b = iqs.QubitRegister(5, "base", 4)
    before = a.GetStateVector()
    sweeps = C.c_uint(99)
    check(lib.iqsg_apply_ops(a._h, None, 0, C.byref(sweeps)))
    assert sweeps.value == 0
    check(lib.iqsg_adjoint_ops(a._h, b._h, None, 0, None, 0, C.byref(sweeps)))
    assert sweeps.value == 0 and np.array_equal(a.GetStateVector(), before)


@pytest.mark.parametrize("precision", ["DP", "SP"])
def test_one_qubit_register_fused_and_tiles(precision):
    import iqs_gb300 as iqs
    r = iqs.QubitRegister(1, "base", 0, precision=precision)
    r.SetTileQubits(13)  # larger than the register: register sweeps are used
    r.TurnOnFusion()
    o = oracle.OracleRegister(1, "base", 0, precision)
    for reg in (r, o):
        reg.ApplyHadamard(0)
        reg.ApplyRotationZ(0, 0.7)
        reg.ApplyT(0)
        reg.ApplyPauliSqrtY(0)
    tol = TOL_DP if precision == "DP" else 2e-6
    assert np.max(np.abs(r.GetStateVector() - o.GetStateVector())) <= tol
    assert abs(r.GetProbability(0) - o.GetProbability(0)) <= tol


def test_adjoint_without_parameters_undoes_gates_on_both_registers():
    import iqs_gb300 as iqs
    from iqs_gb300 import _lib
    from iqs_gb300._lib import check, lib
    rng = np.random.default_rng(8)
    z = rng.standard_normal((2, 2)) + 1j * rng.standard_normal((2, 2))
    u = np.linalg.qr(z)[0]
    psi = iqs.QubitRegister(3, "base", 5)
    lam = iqs.QubitRegister(3, "base", 2)
    p0, l0 = psi.GetStateVector(), lam.GetStateVector()
    psi.Apply1QubitGate(1, u)
    lam.Apply1QubitGate(1, u)
    arr = (_lib.Op * 1)(_op(_lib.OP_1Q, 1, 0, u.conj().T))
    check(lib.iqsg_adjoint_ops(psi._h, lam._h, arr, 1, None, 0, None))
    assert np.max(np.abs(psi.GetStateVector() - p0)) <= TOL_DP
    assert np.max(np.abs(lam.GetStateVector() - l0)) <= TOL_DP


def test_two_qubit_trotter_chain():
    from iqs_gb300.trotter import XXZChain, bond_gate, strang_layers
    J = [1.1]
    chain = XXZChain(2, J, steps=3, precision="DP", checkpoint_every=1)
    e, g = chain.energy_and_grad()
    o = oracle.OracleRegister(2, "base", 2)
    for bonds, tau in strang_layers(2, 0.05, 3):
        for b in bonds:
            o.Apply2QubitGate(1, 0, bond_gate(0.5 * tau * J[b], 0.8))
    assert abs(e - o.ExpectationValue([0, 1], [3, 3], 1.0)) <= TOL_DP
    # <ZZ> is conserved by an XXZ bond from the Neel state |01>: the gradient vanishes
    assert abs(e + 1.0) <= 1e-12 and abs(g[0]) <= 1e-12


def test_single_qubit_batch_instances():
    import iqs_gb300 as iqs
    inst = [(1, 2, [(0.5, "Z"), (1.5, "X")]), (2, 1, [(1.0, "ZZ")]), (1, 1, [(-2.0, "Y")])]
    b = iqs.BatchedAnsatz(inst, precision="DP")
    params = np.random.default_rng(4).uniform(0, 2 * math.pi, b.num_params)
    e, g = b.run(params, with_grad=True)
    for i, (n, L, terms) in enumerate(inst):
        prm = params[b.param_slices()[i]]
        r = oracle.OracleRegister(n, "base", 0)
        for l in range(L):
            for q in range(n):
                r.ApplyRotationZ(q, prm[2 * (l * n + q)])
                r.ApplyRotationY(q, prm[2 * (l * n + q) + 1])
            for q in range(n - 1):
                r.ApplyCPauliZ(q, q + 1)
        want = 0.0
        for c, s in terms:
            qs = [q for q, ch in enumerate(s) if ch != "I"]
            want += r.ExpectationValue(qs, [{"X": 1, "Y": 2, "Z": 3}[s[q]] for q in qs], c)
        assert abs(e[i] - want) <= TOL_DP
    assert np.all(np.isfinite(g))


def test_batch_rejects_bad_instances():
    import iqs_gb300 as iqs
    with pytest.raises(ValueError):
        iqs.BatchedAnsatz([(25, 1, [(1.0, "Z" * 25)])])  # above 24 qubits
    with pytest.raises(ValueError):
        iqs.BatchedAnsatz([(0, 1, [])])
