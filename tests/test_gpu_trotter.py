"""XXZ-chain Trotter evolution and the two-vector adjoint sweeps (iqsg_adjoint_ops).

Forward states and bond correlators are compared with the oracle applying the same bond
gates through Apply2QubitGate; gradients with central differences of oracle energies, and
the checkpointed and plain backward passes with each other. A generic adjoint circuit (RY
rotations + CZ bricks, one-qubit gradient ops) is checked against the parameter-shift rule
on the oracle."""
import ctypes as C
import math

import numpy as np
import pytest

import oracle
from conftest import TOL_DP, TOL_SP

pytestmark = pytest.mark.gpu


def couplings(n, seed=7):
    return np.random.default_rng(seed).uniform(0.5, 1.5, n - 1)


def oracle_state(n, J, delta, dt, steps, precision="DP"):
    from iqs_gb300.trotter import bond_gate, strang_layers
    o = oracle.OracleRegister(n, "base", sum(1 << q for q in range(1, n, 2)), precision)
    for bonds, tau in strang_layers(n, dt, steps):
        for b in bonds:
            o.Apply2QubitGate(b + 1, b, bond_gate(0.5 * tau * J[b], delta))
    return o


def oracle_energy(n, J, delta, dt, steps):
    o = oracle_state(n, J, delta, dt, steps)
    return sum(o.ExpectationValue([b, b + 1], [3, 3], 1.0) for b in range(n - 1))


@pytest.mark.parametrize("precision,tol", [("DP", TOL_DP), ("SP", TOL_SP)])
def test_forward_matches_oracle(precision, tol):
    from iqs_gb300.trotter import XXZChain
    n, steps = 11, 5
    J = couplings(n)
    chain = XXZChain(n, J, steps=steps, precision=precision, checkpoint_every=None)
    zz = chain.bond_zz()
    o = oracle_state(n, J, 0.8, 0.05, steps)
    assert np.max(np.abs(chain.psi.GetStateVector() - o.GetStateVector())) <= tol
    want = [o.ExpectationValue([b, b + 1], [3, 3], 1.0) for b in range(n - 1)]
    assert np.max(np.abs(zz - want)) <= 4 * tol
    gates = sum(len(b) for b, _ in chain.layers())
    # ComplexSP passes hold 4 positions (two bonds); native ComplexDP passes 3 (one bond).
    assert chain.sweeps_forward <= (gates + 1) // 2 + len(chain.layers()) if precision == "SP" else gates


def test_gradient_matches_finite_differences():
    from iqs_gb300.trotter import XXZChain
    n, steps = 8, 4
    J = couplings(n, seed=11)
    chain = XXZChain(n, J, steps=steps, precision="DP", checkpoint_every=None)
    e, g = chain.energy_and_grad()
    assert abs(e - oracle_energy(n, J, 0.8, 0.05, steps)) <= 1e-12
    h = 1e-5
    fd = np.zeros(n - 1)
    for b in range(n - 1):
        jp, jm = J.copy(), J.copy()
        jp[b] += h
        jm[b] -= h
        fd[b] = (oracle_energy(n, jp, 0.8, 0.05, steps) - oracle_energy(n, jm, 0.8, 0.05, steps)) / (2 * h)
    assert np.max(np.abs(g - fd)) <= 1e-8 * max(1.0, np.max(np.abs(fd)))


def test_checkpointed_backward_agrees():
    from iqs_gb300.trotter import XXZChain
    n, steps = 10, 12
    J = couplings(n, seed=12)
    ref = XXZChain(n, J, steps=steps, precision="DP", checkpoint_every=None).energy_and_grad()
    for every in (1, 5, 10):
        chain = XXZChain(n, J, steps=steps, precision="DP", checkpoint_every=every)
        e, g = chain.energy_and_grad()
        assert len(chain._ckpt) == len(range(every, steps, every))
        assert abs(e - ref[0]) <= 1e-13 and np.max(np.abs(g - ref[1])) <= 1e-11


def test_single_precision_gradient():
    from iqs_gb300.trotter import XXZChain
    n, steps = 12, 6
    J = couplings(n, seed=13)
    e64, g64 = XXZChain(n, J, steps=steps, precision="DP").energy_and_grad()
    e32, g32 = XXZChain(n, J, steps=steps, precision="SP", checkpoint_every=2).energy_and_grad()
    assert abs(e32 - e64) <= 1e-5
    assert np.max(np.abs(g32 - g64)) <= 1e-4 * max(1.0, np.max(np.abs(g64)))


def _op(kind, t0, t1=0, m=None, value=0):
    from iqs_gb300 import _lib
    op = _lib.Op()
    op.kind, op.t0, op.t1, op.value = kind, t0, t1, value
    if m is not None:
        a = np.ascontiguousarray(m, dtype=np.complex128).reshape(-1).view(np.float64)
        C.memmove(op.m, a.ctypes.data, a.nbytes)
    return op


def _ry(t):
    c, s = math.cos(t / 2), math.sin(t / 2)
    return np.array([[c, -s], [s, c]], dtype=complex)


@pytest.mark.parametrize("precision", ["DP", "SP"])
def test_generic_one_qubit_gradients_match_parameter_shift(precision):
    """RY(theta_k) on every qubit + CZ bricks, L layers; E = sum_e <Z_u Z_v> on a ring."""
    import iqs_gb300 as iqs
    from iqs_gb300 import _lib
    from iqs_gb300._lib import check, lib
    n, L = 9, 3
    rng = np.random.default_rng(21)
    theta = rng.uniform(-math.pi, math.pi, n * L)
    edges = [(q, (q + 1) % n) for q in range(n)]

    def circuit(reg, th):
        for l in range(L):
            for q in range(n):
                reg.Apply1QubitGate(q, _ry(th[l * n + q]))
            for q in range(l % 2, n - 1, 2):
                reg.ApplyCPauliZ(q, q + 1)

    def oracle_e(th):
        o = oracle.OracleRegister(n, "base", 0)
        circuit(o, th)
        return sum(o.ExpectationValue([u, v], [3, 3], 1.0) for u, v in edges)

    psi = iqs.QubitRegister(n, "base", 0, precision=precision)
    circuit(psi, theta)
    lam = iqs.QubitRegister(n, "", 0, precision=precision)
    e_arr = np.asarray(edges, dtype=np.uint32).reshape(-1)
    en = C.c_double()
    check(lib.iqsg_qaoa_observable(psi._h, lam._h, len(edges), e_arr.ctypes.data_as(_lib._UP), None, C.byref(en), None))
    Y = np.array([[0, -1j], [1j, 0]])
    cz = np.diag([1, 1, 1, -1]).astype(complex)
    ops = []
    for l in range(L - 1, -1, -1):
        for q in reversed(range(l % 2, n - 1, 2)):
            ops.append(_op(_lib.OP_DIAG2, q, q + 1, np.diag(cz)))
        for q in range(n - 1, -1, -1):
            k = l * n + q
            ops.append(_op(_lib.OP_GRAD1, q, 0, Y, value=k))  # RY = exp(-i theta Y / 2): M = 2 * (1/2) Y
            ops.append(_op(_lib.OP_1Q, q, 0, _ry(-theta[k])))
    grads = np.zeros(n * L)
    arr = (_lib.Op * len(ops))(*ops)
    sweeps = C.c_uint()
    check(lib.iqsg_adjoint_ops(psi._h, lam._h, arr, len(arr), grads.ctypes.data_as(_lib._DP), n * L, C.byref(sweeps)))
    assert 0 < sweeps.value < len(ops)
    ps = np.zeros(n * L)
    for k in range(n * L):
        a, b = theta.copy(), theta.copy()
        a[k] += math.pi / 2
        b[k] -= math.pi / 2
        ps[k] = (oracle_e(a) - oracle_e(b)) / 2
    assert abs(en.value - oracle_e(theta)) <= (1e-12 if precision == "DP" else 1e-5)
    assert np.max(np.abs(grads - ps)) <= (1e-11 if precision == "DP" else 2e-5)
    # psi was walked back to |0...0>
    st = psi.GetStateVector()
    assert abs(st[0] - 1) <= (1e-12 if precision == "DP" else 1e-5)


def test_adjoint_ops_reject_bad_input():
    import iqs_gb300 as iqs
    from iqs_gb300 import _lib
    from iqs_gb300._lib import lib
    a = iqs.QubitRegister(6, "base", 0)
    b = iqs.QubitRegister(6, "base", 0)
    c = iqs.QubitRegister(7, "base", 0)
    s = iqs.QubitRegister(6, "base", 0, precision="SP")
    grads = np.zeros(4)
    gp = grads.ctypes.data_as(_lib._DP)
    good = (_lib.Op * 1)(_op(_lib.OP_GRAD1, 0, 0, np.eye(2), value=1))
    assert lib.iqsg_adjoint_ops(a._h, b._h, good, 1, gp, 4, None) == _lib.IQSG_OK
    assert lib.iqsg_adjoint_ops(a._h, a._h, good, 1, gp, 4, None) == _lib.IQSG_EINVAL
    assert lib.iqsg_adjoint_ops(a._h, c._h, good, 1, gp, 4, None) == _lib.IQSG_EINVAL
    assert lib.iqsg_adjoint_ops(a._h, s._h, good, 1, gp, 4, None) == _lib.IQSG_EINVAL
    assert lib.iqsg_adjoint_ops(a._h, b._h, good, 1, gp, 1, None) == _lib.IQSG_EINVAL  # value 1 >= nparams
    assert lib.iqsg_adjoint_ops(a._h, b._h, good, 1, None, 4, None) == _lib.IQSG_EINVAL
    bad = (_lib.Op * 1)(_op(_lib.OP_GRAD2, 3, 3, np.eye(4), value=0))
    assert lib.iqsg_adjoint_ops(a._h, b._h, bad, 1, gp, 4, None) == _lib.IQSG_EINVAL
    assert lib.iqsg_apply_ops(a._h, good, 1, None) == _lib.IQSG_EINVAL  # gradient ops need two registers
    assert b"iqsg_apply_ops" in lib.iqsg_last_error()


@pytest.mark.parametrize("precision,n,tol", [("SP", 26, 1e-4), ("DP", 22, 1e-12)])
def test_round_trip_returns_to_the_neel_state(precision, n, tol):
    """Size-independent check: the circuit followed by its inverse is the identity."""
    from iqs_gb300.trotter import XXZChain
    J = couplings(n, seed=3)
    chain = XXZChain(n, J, steps=8, precision=precision, checkpoint_every=None)
    chain.forward()
    assert abs(chain.psi.ComputeNorm() - 1.0) <= tol
    chain.undo()
    assert abs(abs(chain.psi[chain.neel_index()]) ** 2 - 1.0) <= tol
