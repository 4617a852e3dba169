"""Pin the C restatement (oracle/iqs_oracle.c) against the golden vectors the reference
produced, and -- where the reference is built in this checkout -- against the reference
directly on fresh seeded circuits."""
import numpy as np
import pytest

import oracle
from circuits import random_circuit, random_state, replay
from conftest import REPO, case_meta, case_ops, compare_final, golden_cases

# The restatement uses the same operation order and rounding as the reference's x86 build,
# so DP results agree to the last few ulps; SP results to float round-off.
ORACLE_TOL = {"DP": 1e-14, "SP": 1e-6}


def _run_oracle(store, name):
    meta = case_meta(store, name)
    reg = oracle.OracleRegister(meta["n"], meta["style"], meta["base"], meta["precision"])
    if f"{name}/init" in store:
        reg.SetStateVector(store[f"{name}/init"])
    q = replay(reg, case_ops(store, name))
    return reg, np.asarray(q), meta


def test_golden_file_has_cases(golden):
    assert len(golden_cases(golden)) >= 25


@pytest.mark.parametrize("prefix", ["kat_", "random_", "collapse_", "fusion_", "plain_"])
def test_oracle_matches_reference_golden(golden, prefix):
    names = golden_cases(golden, prefix)
    assert names
    for name in names:
        reg, q, meta = _run_oracle(golden, name)
        tol = ORACLE_TOL[meta["precision"]]
        err = compare_final(golden, name, reg.GetStateVector().astype(np.complex128), tol)
        assert err <= tol, f"{name}: state differs from the reference by {err:.3e}"
        assert reg.perm.map == [int(x) for x in golden[f"{name}/map"]], f"{name}: qubit map differs"
        gq = golden[f"{name}/queries"]
        assert q.shape == gq.shape
        if q.size:
            qerr = float(np.max(np.abs(q - gq)))
            assert qerr <= (1e-13 if meta["precision"] == "DP" else 2e-6), f"{name}: query values differ by {qerr:.3e}"


def test_oracle_swap_kat_exact(golden):
    reg, _, _ = _run_oracle(golden, "kat_swap_3q")
    assert [v.real for v in reg.GetStateVector()] == [0, 4, 2, 6, 1, 5, 3, 7]


@pytest.mark.parametrize("name", ["qaoa_ring6", "qaoa_random10"])
def test_oracle_qaoa_golden(golden, name):
    import json
    meta = json.loads(str(golden[f"{name}/meta"]))
    n = meta["n"]
    diag = oracle.OracleRegister(n, "base", 0)
    mx = oracle.oracle_maxcut_cost(diag, golden[f"{name}/adjacency"])
    assert mx == int(golden[f"{name}/max_cut"])
    assert np.array_equal(diag.GetStateVector().real, golden[f"{name}/cost"])
    psi = oracle.OracleRegister(n, "++++", 0)
    for g, b in zip(meta["gammas"], meta["betas"]):
        oracle.oracle_qaoa_layer(psi, diag, g)
        for q in range(n):
            psi.ApplyRotationX(q, 2 * b)
    assert np.max(np.abs(psi.GetStateVector() - golden[f"{name}/final"])) <= 1e-14
    e = [oracle.oracle_qaoa_expectation(psi, diag, 1), oracle.oracle_qaoa_expectation(psi, diag, 2)]
    assert np.allclose(e, golden[f"{name}/expectation"], rtol=0, atol=1e-12)


@pytest.mark.skipif(not oracle.ref_available(), reason="reference sources not built in this checkout")
@pytest.mark.parametrize("n,prec,seed", [(4, "DP", 101), (7, "DP", 102), (10, "DP", 103), (6, "SP", 104), (9, "SP", 105)])
def test_oracle_matches_reference_fresh(n, prec, seed):
    rng = np.random.default_rng(seed)
    init = random_state(n, rng)
    ops = random_circuit(n, 200, rng)
    a = oracle.OracleRegister(n, "base", 0, prec)
    b = oracle.RefRegister(n, "base", 0, prec)
    a.SetStateVector(init)
    b.SetStateVector(init)
    qa, qb = replay(a, ops), replay(b, ops)
    tol = ORACLE_TOL[prec]
    assert np.max(np.abs(a.GetStateVector().astype(np.complex128) - b.GetStateVector())) <= tol
    assert np.max(np.abs(np.asarray(qa) - np.asarray(qb)), initial=0.0) <= (1e-13 if prec == "DP" else 2e-6)
    assert a.perm.map == b.map


def _qaoa_extra():
    import json
    z = np.load(REPO / "tests" / "golden" / "qaoa_extra.npz")
    for name in sorted({k.split("/")[0] for k in z.files}):
        yield name, json.loads(str(z[f"{name}/meta"])), {k.split("/", 1)[1]: z[k] for k in z.files
                                                         if k.startswith(name + "/")}


def test_oracle_weighted_cost_and_histograms_golden():
    """The C restatement of the weighted cost and the numpy restatement of the histograms
    against the reference's outputs."""
    for name, meta, d in _qaoa_extra():
        n, prec = meta["n"], meta["precision"]
        diag = oracle.OracleRegister(n, "base", 0, prec)
        if meta["weighted"]:
            mx = oracle.oracle_weighted_maxcut_cost(diag, d["adj"])
        else:
            mx = oracle.oracle_maxcut_cost(diag, d["adj"].astype(np.int32))
        assert abs(mx - meta["max_cut"]) <= 1e-12 * max(1, mx), name
        assert np.max(np.abs(diag.GetStateVector() - d["diag"])) <= 1e-12, name
        psi = oracle.OracleRegister(n, "", 0, prec)
        psi.SetStateVector(d["psi"])
        for k, (mode, width) in enumerate(meta["hists"]):
            h = oracle.oracle_cost_histogram(psi, diag, mode, meta["max_cut"], width)
            assert np.max(np.abs(h - d[f"hist{k}"])) <= 1e-12, (name, k)


def test_oracle_google_stats_golden():
    import json
    z = np.load(REPO / "tests" / "golden" / "state_io.npz")
    for name in sorted({k.split("/")[0] for k in z.files}):
        meta = json.loads(str(z[f"{name}/meta"]))
        r = oracle.OracleRegister(meta["n"], "base", 0, meta["precision"])
        r.SetStateVector(z[f"{name}/init"])
        want = z[f"{name}/stats"]
        got = np.asarray(oracle.oracle_google_stats(r))
        tol = 1e-12 if meta["precision"] == "DP" else 1e-5
        assert np.max(np.abs(got - want) / np.maximum(1.0, np.abs(want))) <= tol, name


def test_oracle_random_init_golden():
    """Initialize("rand") restated (numpy MT19937 with the C++ standard library's uniform
    distribution) against the reference's own states."""
    import json
    z = np.load(REPO / "tests" / "golden" / "rand_init.npz")
    for name in sorted({k.split("/")[0] for k in z.files}):
        meta = json.loads(str(z[f"{name}/meta"]))
        n, prec, seed = meta["n"], meta["precision"], meta["seed"]
        stream_seed = seed if meta["base_index"] == 0 else seed + 2  # "pool" or "local" stream
        skip = 2 * (1 << n) * (meta["times"] - 1)
        v = oracle.oracle_uniform_random(stream_seed, skip, 2 * (1 << n), -1.0, 1.0, prec).astype(np.float64)
        st = v[0::2] + 1j * v[1::2]
        st /= np.linalg.norm(st)
        tol = 1e-14 if prec == "DP" else 1e-6
        assert np.max(np.abs(st - z[f"{name}/state"])) <= tol, name
