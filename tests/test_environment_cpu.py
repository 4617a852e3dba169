"""The pool-of-states environment (EnvInit / MPIEnvironment) on the CPU: one process, and two
gloo ranks started by EnvInit from a launcher's environment, each rank one state."""
import os
import socket
import sys

import pytest

from conftest import REPO

pytest.importorskip("torch")


def test_single_process_pool():
    import iqs_gb300 as iqs
    iqs.EnvInit()
    E = iqs.MPIEnvironment
    assert (E.GetRank(), E.GetSizeWorldComm(), E.GetPoolRank(), E.GetPoolSize()) == (0, 1, 0, 1)
    assert (E.GetStateRank(), E.GetStateSize(), E.GetStateId(), E.GetNumStates()) == (0, 1, 0, 1)
    assert E.IsUsefulRank() and E.GetNumNodes() == 1
    assert E.IncoherentSumOverAllStatesOfPool(0.25) == 0.25
    E.Barrier()
    E.StateBarrier()
    E.UpdateStateComm(1)
    with pytest.raises(ValueError):
        E.UpdateStateComm(2)
    iqs.EnvFinalizeDummyRanks()
    iqs.EnvFinalize()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port),
                      LOCAL_WORLD_SIZE=str(world))
    sys.path.insert(0, str(REPO / "intel-qs_gb300"))
    import iqs_gb300 as iqs
    iqs.EnvInit()
    E = iqs.MPIEnvironment
    try:
        E.Barrier()
        total = E.IncoherentSumOverAllStatesOfPool(float(E.GetStateId() + 1))
        q.put((E.GetRank(), E.GetStateId(), E.GetNumStates(), E.GetStateSize(), E.GetNumNodes(), total))
    finally:
        iqs.EnvFinalize()


def test_two_ranks_are_two_states():
    """NoisySimulationTest.OneStatePerRank's layout (noisy_simulation_test.hpp:132-170): each rank
    one state, pool sums over the states."""
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    assert got == [(0, 0, 2, 1, 1, 3.0), (1, 1, 2, 1, 1, 3.0)]


def _rng_rank(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, str(REPO / "intel-qs_gb300"))
    sys.path.insert(0, str(REPO))
    import iqs_gb300 as iqs
    import oracle
    iqs.EnvInit()
    try:
        rng = iqs.RandomNumberGenerator()
        rng.SetSeedStreamPtrs(777)
        got = {s: list(rng.UniformRandomNumbers(5, 0, 1, s)) for s in ("pool", "state", "local")}
        want = {"pool": 777, "state": 777 + 1 + rank, "local": 777 + 1 + world + rank}
        ok = all(list(oracle.oracle_uniform_random(want[s], 0, 5, 0.0, 1.0, "DP")) == got[s] for s in got)
        q.put((rank, ok, got["pool"][0]))
    finally:
        iqs.EnvFinalize()


def test_stream_seeds_follow_the_pool():
    """SetSeedStreamPtrs in a pool of two one-state ranks (src/rng_utils.cpp:84-99): the pool
    stream is shared, the state and local streams are seeded by state id and pool rank."""
    import torch.multiprocessing as mp
    oracle_path = str(REPO)
    if oracle_path not in sys.path:
        sys.path.insert(0, oracle_path)
    import oracle
    oracle.build(ref=False)
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rng_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    assert [g[1] for g in got] == [True, True]
    assert got[0][2] == got[1][2]  # the pool stream is common to the pool


def test_intelqs_py_module_name():
    """Programs that `import intelqs_py as iqs` find every name the reference's module binds
    (pybind11/intelqs_py.cpp), apart from the MKL-only SetRndStreamPtrs."""
    sys.path.insert(0, str(REPO / "intel-qs_gb300"))
    import intelqs_py as iqs
    for name in ("QubitRegister", "RandomNumberGenerator", "CM4x4", "CM16x16", "MPIEnvironment", "EnvInit",
                 "EnvFinalize", "EnvFinalizeDummyRanks", "InitializeVectorAsMaxCutCostFunction",
                 "ImplementQaoaLayerBasedOnCostFunction", "GetExpectationValueFromCostFunction",
                 "GetHistogramFromCostFunctionWithWeightsBinned"):
        assert hasattr(iqs, name), name
