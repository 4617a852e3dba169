"""Batched uneven circuits (one persistent launch, CUDA graph): energies against the oracle
running each instance gate by gate, gradients against the parameter-shift rule on the oracle."""
import math

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def _instances(count, rng, nmin=3, nmax=7, lmax=3, nterms=3):
    out = []
    for _ in range(count):
        n = int(rng.integers(nmin, nmax + 1))
        L = int(rng.integers(1, lmax + 1))
        terms = [(float(rng.standard_normal()), "".join(rng.choice(list("IXYZ"), size=n))) for _ in range(nterms)]
        out.append((n, L, terms))
    return out


def _oracle_energy(n, L, terms, prm, prec):
    r = oracle.OracleRegister(n, "base", 0, prec)
    for l in range(L):
        for q in range(n):
            r.ApplyRotationZ(q, prm[2 * (l * n + q)])
            r.ApplyRotationY(q, prm[2 * (l * n + q) + 1])
        for q in range(n - 1):
            r.ApplyCPauliZ(q, q + 1)
    e = 0.0
    for c, s in terms:
        qs = [q for q, ch in enumerate(s) if ch != "I"]
        obs = [{"X": 1, "Y": 2, "Z": 3}[s[q]] for q in qs]
        e += r.ExpectationValue(qs, obs, c) if qs else c
    return e


@pytest.mark.parametrize("prec,tol", [("DP", 1e-12), ("SP", 2e-5)])
def test_batched_energies_and_gradients(prec, tol):
    import iqs_gb300 as iqs
    rng = np.random.default_rng(55)
    inst = _instances(12, rng)
    b = iqs.BatchedAnsatz(inst, precision=prec)
    params = rng.uniform(0, 2 * math.pi, b.num_params)
    e, g = b.run(params, with_grad=True)
    for i, (n, L, terms) in enumerate(inst):
        prm = params[b.param_slices()[i]]
        assert abs(e[i] - _oracle_energy(n, L, terms, prm, "DP")) <= tol * max(1.0, sum(abs(c) for c, _ in terms))
        if i < 4:  # parameter shift (pi/2) on the oracle for every parameter of a few instances
            ps = np.zeros(prm.size)
            for k in range(prm.size):
                a, z = prm.copy(), prm.copy()
                a[k] += math.pi / 2
                z[k] -= math.pi / 2
                ps[k] = (_oracle_energy(n, L, terms, a, "DP") - _oracle_energy(n, L, terms, z, "DP")) / 2
            scale = max(1.0, np.max(np.abs(ps)))
            assert np.max(np.abs(g[b.param_slices()[i]] - ps)) / scale <= (1e-10 if prec == "DP" else 5e-4)
    # graph replay: same inputs, same outputs; new inputs, fresh results
    e2, g2 = b.run(params, with_grad=True)
    assert np.array_equal(e, e2) and np.array_equal(g, g2)
    e_only = b.run(params)
    assert np.array_equal(e_only, e)
    p3 = rng.uniform(0, 2 * math.pi, b.num_params)
    e3 = b.run(p3)
    n, L, terms = inst[0]
    assert abs(e3[0] - _oracle_energy(n, L, terms, p3[b.param_slices()[0]], "DP")) <= tol * 10


def test_batched_launch_shapes_agree():
    import iqs_gb300 as iqs
    rng = np.random.default_rng(66)
    inst = _instances(40, rng, nmin=6, nmax=13, lmax=4, nterms=4)
    b = iqs.BatchedAnsatz(inst, precision="SP")
    params = rng.uniform(0, 2 * math.pi, b.num_params)
    ref_e, ref_g = b.run(params, with_grad=True)
    table = b.autotune(params, shapes=((128, 4), (512, 2), (256, 4)), trials=1)
    assert len(table) == 3
    e, g = b.run(params, with_grad=True)
    assert np.max(np.abs(e - ref_e)) <= 1e-6 and np.max(np.abs(g - ref_g)) <= 1e-5
