"""iqsg_probability_static: the measurement entry point that allocates nothing.

It serves callers that cannot allocate device memory when they measure (HBM already
filled by their registers, no implicit device-wide synchronisation allowed, or a framework
that owns all device memory). The test calls it through the C ABI on a register's device
amplitudes, twice in a row (the static scratch keeps the previous call's contents), and
compares each result with iqsg_probability, the allocating entry point. This file is named
so that pytest collects it last.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import TOL_DP, TOL_SP

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", ["DP", "SP"])
def test_static_probability_matches_allocating_entry_point(prec):
    torch = pytest.importorskip("torch")
    import iqs_gb300
    from iqs_gb300._lib import check, lib

    n = 20
    rng = np.random.default_rng(9090)
    v = rng.standard_normal(1 << n) + 1j * rng.standard_normal(1 << n)
    v /= np.linalg.norm(v)
    reg = iqs_gb300.QubitRegister(n, "base", 0, precision=prec)
    reg.SetStateVector(v)
    reg.synchronize()
    amps = reg.RawState()
    p_code = 0 if prec == "DP" else 1
    out = torch.full((2,), -1.0, dtype=torch.float64, device="cuda")
    tol = TOL_DP if prec == "DP" else TOL_SP
    for call, pos in enumerate((3, 17)):  # two calls in a row share the static scratch
        expected = C.c_double()
        check(lib.iqsg_probability(reg._h, pos, C.byref(expected)))
        dst = C.c_void_p(out.data_ptr() + 8 * call)
        check(lib.iqsg_probability_static(C.c_void_p(amps), n, p_code, pos, dst, None))
        torch.cuda.synchronize()
        got = float(out[call].item())
        assert abs(got - expected.value) <= tol, (call, got, expected.value)


def test_static_probability_rejects_bad_sizes():
    from iqs_gb300._lib import IQSG_EINVAL, lib

    dummy = C.c_void_p(256)
    res = C.c_void_p(512)
    assert lib.iqsg_probability_static(dummy, 41, 0, 0, res, None) == IQSG_EINVAL
    assert b"num_qubits" in lib.iqsg_last_error()
    assert lib.iqsg_probability_static(dummy, 10, 0, 10, res, None) == IQSG_EINVAL
    assert lib.iqsg_probability_static(None, 10, 0, 0, res, None) == IQSG_EINVAL
