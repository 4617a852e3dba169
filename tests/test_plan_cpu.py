"""The fusion plan of iqsg_apply_ops computed on the host (iqsg_plan_ops, no GPU): how the
scheduler packs the bench's gate layer and other streams into passes."""
import numpy as np
import pytest

from circuits import haar_2x2


def _layer_ops(n, rng):
    from iqs_gb300 import _lib
    from iqs_gb300.qureg import _m2, _op
    ops = [_op(_lib.OP_1Q, q, 0, _m2(haar_2x2(rng))) for q in range(n)]
    cz = _m2([[1, 0], [0, -1]])
    ops += [_op(_lib.OP_CTRL, 2 * j + 1, 0, cz, ctrl=(2 * j,)) for j in range(n // 2)]
    ops += [_op(_lib.OP_CTRL, 2 * j + 2, 0, cz, ctrl=(2 * j + 1,)) for j in range((n - 1) // 2)]
    return ops


def test_headline_layer_plan():
    """The 30-qubit layer (Haar U on every qubit + CZ brick): 15 two-qubit passes in emulated
    ComplexDP, the whole brick as diagonal operations of the last pass, run as double-float
    pairs; 10 passes at width 3 (native FP64), 8 at width 4 (ComplexSP)."""
    from iqs_gb300.qureg import plan_ops
    ops = _layer_ops(30, np.random.default_rng(1))
    p = plan_ops(30, ops, precision="DP", math="emulated")
    assert len(p["sweeps"]) == 15 and p["pair_storage"]
    assert all(s["k"] == 2 and s["one_qubit"] == 2 for s in p["sweeps"])
    assert [s["diagonal"] > 0 for s in p["sweeps"]] == [False] * 14 + [True]
    assert sorted(q for s in p["sweeps"] for q in s["positions"]) == list(range(30))
    assert len(plan_ops(30, ops, precision="DP", math="native")["sweeps"]) == 10
    assert not plan_ops(30, ops, precision="DP", math="native")["pair_storage"]
    assert len(plan_ops(30, ops, precision="SP")["sweeps"]) == 8
    assert len(plan_ops(30, ops, precision="DP", math="emulated", width=1)["sweeps"]) == 30


def test_plan_rules_for_pairs():
    from iqs_gb300 import _lib
    from iqs_gb300.qureg import _m2, _op, plan_ops
    rng = np.random.default_rng(2)
    ops = _layer_ops(12, rng)
    assert plan_ops(12, ops[:3], precision="DP", math="emulated")["pair_storage"] is False  # 2 sweeps
    big = ops + [_op(_lib.OP_1Q, 4, 0, _m2(1.5 * haar_2x2(rng)))]
    assert plan_ops(12, big, precision="DP", math="emulated")["pair_storage"] is False  # not contractive
    assert plan_ops(12, [], precision="DP", math="emulated") == {"sweeps": [], "pair_storage": False}


def test_plan_rejects_bad_input():
    from iqs_gb300 import _lib
    from iqs_gb300.qureg import _m2, _op, plan_ops
    with pytest.raises(ValueError):
        plan_ops(4, [_op(_lib.OP_1Q, 7, 0, _m2(np.eye(2)))])  # position beyond the register
    with pytest.raises(ValueError):
        plan_ops(4, [], width=9)
