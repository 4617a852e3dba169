"""Emulated-ComplexDP fused sweeps with a share of the warps on native FP64
(IQSG_OPT_NATIVE_SHARE): every share agrees with the oracle at the DP bar."""
import numpy as np
import pytest

import oracle
from circuits import brick_layer_ops, replay
from conftest import TOL_DP

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("share", [0, 3, 8, 16])
@pytest.mark.parametrize("width", [1, 2, 3])
def test_native_share(share, width):
    import iqs_gb300 as iqs
    n = 18
    rng = np.random.default_rng(31)
    ops = []
    for _ in range(3):
        ops += brick_layer_ops(n, rng, "ApplyCPauliZ")
    reg = iqs.QubitRegister(n, "base", 77, math="emulated")
    reg.SetSweepWidth(width)
    reg.SetNativeShare(share)
    reg.TurnOnFusion()
    replay(reg, ops)
    reg.ApplyFusedGates()
    ref = oracle.OracleRegister(n, "base", 77)
    replay(ref, ops)
    assert np.max(np.abs(reg.GetStateVector() - ref.GetStateVector())) <= TOL_DP


def test_native_share_rejects_out_of_range():
    import iqs_gb300 as iqs
    reg = iqs.QubitRegister(4, "base", 0, math="emulated")
    with pytest.raises(ValueError):
        reg.SetNativeShare(17)
