"""QFT followed by 40 Haar/CZ brick layers (examples/quantum_fourier_transform.cpp:49-71 for
the QFT gate order), from a seeded basis state: ComplexDP gate by gate in native and emulated
arithmetic, and ComplexSP in fused passes, against amplitudes the reference itself computed
(tests/golden/qft_brick.npz). The SP run is also compared with the DP run over the whole
state (max abs difference and fidelity |<psi_DP|psi_SP>|^2)."""
import hashlib
import json

import numpy as np
import pytest

from circuits import loads, qft_brick_queries, replay
from conftest import REPO, TOL_DP

pytestmark = pytest.mark.gpu

FIXTURE = REPO / "tests" / "golden" / "qft_brick.npz"

# ComplexSP bars after ~2.2k gates (unit roundoff 6e-8 per operation): per-amplitude error
# relative to the typical amplitude 2^-n/2, and infidelity against the FP64 result.
SP_REL_AMP = 2e-4
SP_INFIDELITY = 1e-8


def load_case(n):
    z = np.load(FIXTURE)
    if f"n{n}/meta" not in z.files:
        pytest.skip(f"no {n}-qubit case in the fixture")
    meta = json.loads(str(z[f"n{n}/meta"]))
    text = str(z[f"n{n}/ops"])
    assert hashlib.sha256(text.encode()).hexdigest() == meta["ops_sha256"]
    return meta, loads(text), z[f"n{n}/idx"], z[f"n{n}/amps"], z[f"n{n}/queries"]


def device_view(reg):
    import torch
    return torch.as_tensor(reg, device="cuda")


def compare_full(a_reg, b_reg, chunk=1 << 26):
    """(max |a - b|, |<a|b>|^2 / (<a|a><b|b>)) over the whole state, in FP64 on the device."""
    import torch
    a, b = device_view(a_reg), device_view(b_reg)
    mx, ov, na, nb = 0.0, 0j, 0.0, 0.0
    for s in range(0, a.numel(), chunk):
        x = a[s:s + chunk].to(torch.complex128)
        y = b[s:s + chunk].to(torch.complex128)
        mx = max(mx, float((x - y).abs().max()))
        ov += complex(torch.vdot(x, y))
        na += float(torch.vdot(x, x).real)
        nb += float(torch.vdot(y, y).real)
    return mx, abs(ov) ** 2 / (na * nb)


def run(n, ops, start, precision, math="native", fusion=False):
    import iqs_gb300 as iqs
    reg = iqs.QubitRegister(n, "base", start, precision=precision, math=math)
    if fusion:
        reg.TurnOnFusion()
    replay(reg, ops)
    sweeps = reg.ApplyFusedGates() if fusion else 0
    reg.synchronize()
    return reg, sweeps


def sampled(reg, idx):
    import torch
    return device_view(reg)[torch.as_tensor(idx, device="cuda")].cpu().numpy().astype(np.complex128)


@pytest.mark.parametrize("n", [24, 30])
def test_qft_brick_against_reference(n):
    meta, ops, idx, amps, queries = load_case(n)
    scale = 2.0 ** (-n / 2)
    dp = {}
    for math in ("emulated", "native"):
        reg, _ = run(n, ops, meta["start"], "DP", math)
        assert np.max(np.abs(sampled(reg, idx) - amps)) <= TOL_DP
        got = replay(reg, qft_brick_queries(n))
        assert np.max(np.abs(np.asarray(got) - queries)) <= TOL_DP
        if math == "emulated":
            dp = reg
        else:
            mx, fid = compare_full(dp, reg)
            assert mx <= TOL_DP and 1.0 - fid <= 1e-12
            del reg
    sp, sweeps = run(n, ops, meta["start"], "SP", fusion=True)
    assert 0 < sweeps < len(ops) // 2
    assert np.max(np.abs(sampled(sp, idx) - amps)) <= SP_REL_AMP * scale
    mx, fid = compare_full(dp, sp)
    assert mx <= SP_REL_AMP * scale and 1.0 - fid <= SP_INFIDELITY
    got = replay(sp, qft_brick_queries(n))
    assert np.max(np.abs(np.asarray(got) - queries)) <= 1e-5
