"""Adjoint-mode QAOA gradients against the FP64 parameter-shift rule on the oracle, central
finite differences on the GPU, the reference's own QAOA route, and torch autograd."""
import math

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def _graph(n, seed, p_edge=0.45):
    rng = np.random.default_rng(seed)
    edges = [(u, v) for u in range(n) for v in range(u + 1, n) if rng.random() < p_edge]
    return edges


def _oracle_energy(n, edges, gam, bet):
    """gam[l][e], bet[l][q]: per-occurrence angles; exp(-i g Z_u Z_v / 2) as ApplyDiag, RX(2 b)."""
    r = oracle.OracleRegister(n, "++++", 0)
    for l in range(len(gam)):
        for e, (u, v) in enumerate(edges):
            a, b = np.exp(-0.5j * gam[l][e]), np.exp(0.5j * gam[l][e])
            r.ApplyDiag(u, v, np.diag([a, b, b, a]))
        for q in range(n):
            r.ApplyRotationX(q, 2 * bet[l][q])
    return sum(r.ExpectationValue([u, v], [3, 3]) for u, v in edges)


def _parameter_shift(n, edges, gammas, betas):
    p = len(gammas)
    gam = [[g] * len(edges) for g in gammas]
    bet = [[b] * n for b in betas]
    dg, db = np.zeros(p), np.zeros(p)
    for l in range(p):
        for e in range(len(edges)):
            gp = [row[:] for row in gam]
            gm = [row[:] for row in gam]
            gp[l][e] += math.pi / 2
            gm[l][e] -= math.pi / 2
            dg[l] += (_oracle_energy(n, edges, gp, bet) - _oracle_energy(n, edges, gm, bet)) / 2
        for q in range(n):
            bp = [row[:] for row in bet]
            bm = [row[:] for row in bet]
            bp[l][q] += math.pi / 4
            bm[l][q] -= math.pi / 4
            db[l] += _oracle_energy(n, edges, gam, bp) - _oracle_energy(n, edges, gam, bm)
    return dg, db


@pytest.fixture(scope="module")
def iqs():
    import iqs_gb300
    return iqs_gb300


@pytest.mark.parametrize("checkpoint", [False, True])
def test_adjoint_matches_parameter_shift(iqs, checkpoint):
    n, p = 8, 3
    edges = _graph(n, 3)
    rng = np.random.default_rng(4)
    gammas, betas = rng.uniform(0, math.pi, p), rng.uniform(0, math.pi, p)
    circ = iqs.QaoaMaxCut(n, edges, checkpoint=checkpoint)
    e, dg, db = circ.energy_and_grad(gammas, betas)
    e_ref = _oracle_energy(n, edges, [[g] * len(edges) for g in gammas], [[b] * n for b in betas])
    assert abs(e - e_ref) <= 1e-12
    pdg, pdb = _parameter_shift(n, edges, gammas, betas)
    scale = max(np.max(np.abs(pdg)), np.max(np.abs(pdb)))
    assert np.max(np.abs(dg - pdg)) / scale <= 1e-8
    assert np.max(np.abs(db - pdb)) / scale <= 1e-8
    # central differences (h = 1e-6) agree to their truncation / round-off error
    fdg, fdb = circ.finite_difference_grad(gammas, betas, h=1e-6)
    assert np.max(np.abs(np.concatenate([fdg - dg, fdb - db]))) / scale <= 1e-6


@pytest.mark.parametrize("n", [13, 17])
def test_adjoint_larger_registers_vs_finite_differences(iqs, n):
    edges = [(q, (q + 1) % n) for q in range(n)] + [(q, (q + 5) % n) for q in range(0, n, 3)]
    rng = np.random.default_rng(n)
    gammas, betas = rng.uniform(0, math.pi, 2), rng.uniform(0, math.pi, 2)
    circ = iqs.QaoaMaxCut(n, edges)
    e, dg, db = circ.energy_and_grad(gammas, betas)
    # after the backward sweep psi is back at |+>^n
    v = circ.psi.GetStateVector()
    assert np.max(np.abs(v - 1 / math.sqrt(1 << n))) <= 1e-12
    fdg, fdb = circ.finite_difference_grad(gammas, betas, h=1e-5)
    scale = max(np.max(np.abs(fdg)), np.max(np.abs(fdb)), 1.0)
    assert np.max(np.abs(np.concatenate([fdg - dg, fdb - db]))) / scale <= 1e-6


def test_adjoint_single_precision(iqs):
    n, p = 10, 2
    edges = _graph(n, 5)
    rng = np.random.default_rng(6)
    gammas, betas = rng.uniform(0, math.pi, p), rng.uniform(0, math.pi, p)
    e64, dg64, db64 = iqs.QaoaMaxCut(n, edges).energy_and_grad(gammas, betas)
    e32, dg32, db32 = iqs.QaoaMaxCut(n, edges, precision="SP").energy_and_grad(gammas, betas)
    assert abs(e32 - e64) <= 1e-4 * max(1, abs(e64))
    assert np.max(np.abs(np.concatenate([dg32 - dg64, db32 - db64]))) <= 1e-4 * max(1, np.max(np.abs(dg64)))


def test_qaoa_layer_matches_reference_route(iqs):
    """Same energy as the reference's route: MaxCut cost vector + ImplementQaoaLayerBasedOnCostFunction
    + ApplyRotationX. exp(-i g H_C) = exp(-i g W/2) exp(+i g cut): the reference angle is -g."""
    n = 9
    edges = _graph(n, 8)
    adj = np.zeros((n, n), dtype=np.int32)
    for u, v in edges:
        adj[u, v] = adj[v, u] = 1
    gammas, betas = [0.37, 1.1], [0.8, 0.25]
    e = iqs.QaoaMaxCut(n, edges).energy(gammas, betas)
    diag = iqs.QubitRegister(n, "base", 0)
    iqs.InitializeVectorAsMaxCutCostFunction(diag, adj.reshape(-1))
    psi = iqs.QubitRegister(n, "++++", 0)
    for g, b in zip(gammas, betas):
        iqs.ImplementQaoaLayerBasedOnCostFunction(psi, diag, -g)
        for q in range(n):
            psi.ApplyRotationX(q, 2 * b)
    cut = iqs.GetExpectationValueFromCostFunction(psi, diag)
    assert abs(e - (len(edges) - 2 * cut)) <= 1e-12


@pytest.mark.parametrize("n", [12, 17])
def test_checkpointed_equals_plain_adjoint(iqs, n):
    edges = [(q, (q + 1) % n) for q in range(n)] + [(q, (q + 4) % n) for q in range(0, n, 2)]
    rng = np.random.default_rng(100 + n)
    gammas, betas = rng.uniform(0, math.pi, 3), rng.uniform(0, math.pi, 3)
    e0, dg0, db0 = iqs.QaoaMaxCut(n, edges).energy_and_grad(gammas, betas)
    e1, dg1, db1 = iqs.QaoaMaxCut(n, edges, checkpoint=True).energy_and_grad(gammas, betas)
    assert abs(e0 - e1) <= 1e-12
    assert np.max(np.abs(np.concatenate([dg0 - dg1, db0 - db1]))) <= 1e-11


def test_torch_autograd(iqs):
    torch = pytest.importorskip("torch")
    n, p = 9, 2
    edges = _graph(n, 9)
    circ = iqs.QaoaMaxCut(n, edges)
    prm = torch.tensor([0.3, 1.2, 0.7, 0.4], dtype=torch.float64, requires_grad=True)
    loss = iqs.qaoa_energy(prm, circ)
    loss.backward()
    _, dg, db = circ.energy_and_grad([0.3, 1.2], [0.7, 0.4])
    assert np.max(np.abs(prm.grad.numpy() - np.concatenate([dg, db]))) <= 1e-12
