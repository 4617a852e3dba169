"""Weighted MaxCut cost vector and cost histograms on the GPU against the reference's own
outputs (tests/golden/qaoa_extra.npz, made by tests/golden/make_qaoa_extra.py), including the
checks of unit_test/include/qaoa_features_test.hpp (histogram mean = expectation)."""
import json

import numpy as np
import pytest

from conftest import REPO

pytestmark = pytest.mark.gpu

FIX = REPO / "tests" / "golden" / "qaoa_extra.npz"


def cases():
    z = np.load(FIX)
    return sorted({k.split("/")[0] for k in z.files})


def load(name):
    z = np.load(FIX)
    return json.loads(str(z[f"{name}/meta"])), {k.split("/", 1)[1]: z[k] for k in z.files if k.startswith(name + "/")}


@pytest.mark.parametrize("name", cases())
def test_cost_vector_layers_and_histograms(name):
    import iqs_gb300 as iqs
    meta, d = load(name)
    n, prec = meta["n"], meta["precision"]
    tol = 1e-12 if prec == "DP" else 2e-5
    diag = iqs.QubitRegister(n, "base", 0, precision=prec)
    adj = d["adj"].reshape(n, n)
    if meta["weighted"]:
        mx = iqs.InitializeVectorAsWeightedMaxCutCostFunction(diag, adj.reshape(-1))
    else:
        mx = iqs.InitializeVectorAsMaxCutCostFunction(diag, adj.astype(np.int32).reshape(-1))
    assert abs(mx - meta["max_cut"]) <= (1e-12 if prec == "DP" else 1e-5) * max(1.0, meta["max_cut"])
    assert np.max(np.abs(diag.GetStateVector() - d["diag"])) <= (1e-12 if prec == "DP" else 1e-5) * meta["max_cut"]
    psi = iqs.QubitRegister(n, "++++", 0, precision=prec)
    for g, b in zip(meta["gammas"], meta["betas"]):
        iqs.ImplementQaoaLayerBasedOnCostFunction(psi, diag, g)
        for q in range(n):
            psi.ApplyRotationX(q, b)
    assert np.max(np.abs(psi.GetStateVector() - d["psi"])) <= tol
    e = iqs.GetExpectationValueFromCostFunction(psi, diag)
    assert abs(e - meta["expectation"]) <= tol * max(1.0, meta["max_cut"])
    funcs = {0: lambda w: iqs.GetHistogramFromCostFunction(psi, diag, int(meta["max_cut"])),
             1: lambda w: iqs.GetHistogramFromCostFunctionWithWeightsRounded(psi, diag, meta["max_cut"]),
             2: lambda w: iqs.GetHistogramFromCostFunctionWithWeightsBinned(psi, diag, meta["max_cut"], w)}
    for k, (mode, width) in enumerate(meta["hists"]):
        h = np.asarray(funcs[mode](width))
        want = d[f"hist{k}"]
        assert h.shape == want.shape
        assert np.max(np.abs(h - want)) <= 1e-12
        assert abs(h.sum() - 1.0) <= 1e-12
        scale = 1.0 if mode < 2 else width
        mean = float(np.sum(np.arange(h.size) * scale * h))
        # integer costs: the mean is the expectation; weighted: below it by less than one bin
        if mode == 0:
            assert abs(mean - e) <= 1e-12
        else:
            assert -1e-12 <= e - mean <= scale + 1e-7


def test_histogram_range_and_order_errors():
    import iqs_gb300 as iqs
    n = 6
    ring = [[1 if abs(i - j) in (1, 5) else 0 for j in range(n)] for i in range(n)]
    diag = iqs.QubitRegister(n, "base", 0)
    mx = iqs.InitializeVectorAsMaxCutCostFunction(diag, np.asarray(ring, dtype=np.int32).reshape(-1))
    psi = iqs.QubitRegister(n, "++++", 0)
    assert len(iqs.GetHistogramFromCostFunction(psi, diag, mx)) == mx + 1
    with pytest.raises(ValueError):  # costs above max_value: the reference asserts
        iqs.GetHistogramFromCostFunction(psi, diag, mx - 2)
    with pytest.raises(ValueError):
        iqs.GetHistogramFromCostFunctionWithWeightsBinned(psi, diag, float(mx), 0.0)
    psi.EmulateSwap(0, 1)
    with pytest.raises(ValueError):  # different qubit orders
        iqs.GetHistogramFromCostFunction(psi, diag, mx)
    bad = np.asarray(ring, dtype=np.float64)
    bad[0, 1] = 2.0  # not symmetric
    with pytest.raises(ValueError):
        iqs.InitializeVectorAsWeightedMaxCutCostFunction(diag, bad.reshape(-1))
