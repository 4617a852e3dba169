"""Host-side pieces of the XXZ Trotter driver: the closed-form bond gate against the matrix
exponential and against RXX RYY RZZ, and the Strang layer list."""
import math

import numpy as np
import scipy.linalg

from iqs_gb300.trotter import bond_gate, bond_generator, strang_layers

X = np.array([[0, 1], [1, 0]], dtype=complex)
Y = np.array([[0, -1j], [1j, 0]], dtype=complex)
Z = np.diag([1.0, -1.0]).astype(complex)


def test_bond_gate_closed_form():
    rng = np.random.default_rng(3)
    for _ in range(20):
        theta, delta = rng.uniform(-2, 2), rng.uniform(-1.5, 1.5)
        A = bond_generator(delta)
        assert np.allclose(A, np.kron(X, X) + np.kron(Y, Y) + delta * np.kron(Z, Z), atol=0)
        G = bond_gate(theta, delta)
        assert np.max(np.abs(G - scipy.linalg.expm(-1j * theta * A))) < 1e-14
        # RXX(2 theta) RYY(2 theta) RZZ(2 delta theta) with R_PP(phi) = exp(-i phi/2 P P)
        rxx = scipy.linalg.expm(-1j * theta * np.kron(X, X))
        ryy = scipy.linalg.expm(-1j * theta * np.kron(Y, Y))
        rzz = scipy.linalg.expm(-1j * theta * delta * np.kron(Z, Z))
        assert np.max(np.abs(G - rxx @ ryy @ rzz)) < 1e-14
        assert np.max(np.abs(G @ bond_gate(-theta, delta) - np.eye(4))) < 1e-14


def test_strang_layers_merge_half_steps():
    L = strang_layers(6, 0.05, 3)
    assert [tau for _, tau in L] == [0.025, 0.05, 0.05, 0.05, 0.05, 0.05, 0.025]
    assert L[0][0] == [0, 2, 4] and L[1][0] == [1, 3]
    # total time per bond: every bond evolves for steps * dt
    for b in range(5):
        t = sum(tau for bonds, tau in L if b in bonds)
        assert math.isclose(t, 3 * 0.05)
