"""Queued host <-> HBM copies (iqsg_upload_async / iqsg_download_async) run in stream order
with the register's gates, and two registers on their own streams do not interfere."""
import numpy as np
import pytest

import oracle
from circuits import brick_layer_ops, replay
from conftest import TOL_DP

pytestmark = pytest.mark.gpu


def test_async_round_trip_in_stream_order():
    import torch
    import iqs_gb300 as iqs
    n = 16
    rng = np.random.default_rng(3)
    ops = brick_layer_ops(n, rng, "ApplyCPauliZ")
    init = rng.standard_normal(1 << n) + 1j * rng.standard_normal(1 << n)
    init /= np.linalg.norm(init)
    ref = oracle.OracleRegister(n, "", 0)
    ref.SetStateVector(init)
    replay(ref, ops)
    want = ref.GetStateVector()
    streams = [torch.cuda.Stream(), torch.cuda.Stream()]
    regs = [iqs.QubitRegister(n, "", 0, stream=s.cuda_stream) for s in streams]
    hosts = [torch.empty(1 << n, dtype=torch.complex128, pin_memory=True).numpy() for _ in regs]
    for step in range(4):
        r, h = regs[step % 2], hosts[step % 2]
        h[:] = init
        r.TurnOnFusion()
        r.SetStateVectorAsync(h)
        replay(r, ops)
        r.GetStateVectorAsync(h)
    for r in regs:
        r.synchronize()
    for h in hosts:
        assert np.max(np.abs(h - want)) <= TOL_DP


def test_async_copies_reject_bad_arrays():
    import iqs_gb300 as iqs
    r = iqs.QubitRegister(6, "base", 0)
    with pytest.raises(ValueError):
        r.SetStateVectorAsync(np.zeros(64, dtype=np.complex64))
    with pytest.raises(ValueError):
        r.GetStateVectorAsync(np.zeros(32, dtype=np.complex128))
