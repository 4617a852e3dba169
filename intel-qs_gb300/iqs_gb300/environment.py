"""The process environment of intel-qs's Python module (pybind11/intelqs_py.cpp:37-66,
397-424; include/mpi_env.hpp): EnvInit / EnvFinalize / EnvFinalizeDummyRanks and the static
MPIEnvironment queries, for this engine's layout: every process drives one GPU and holds one
whole state, so a job of P processes is a pool of P states, each on a single rank (state rank 0,
state size 1, state id = pool rank). That is the reference's "one state per rank" pool
(unit_test/include/noisy_simulation_test.hpp:132-170), the form its noisy-trajectory averages
use. A state split across processes (fewer states than ranks) is not offered.

Ranks come from torch.distributed: EnvInit starts a gloo process group when the launcher set
RANK / WORLD_SIZE (torchrun) and none is running; a single process needs nothing. Pool sums and
barriers go through that group (host values, so gloo on the CPU).
"""
from __future__ import annotations

import os

_OWN_GROUP = False


def _dist():
    try:
        import torch.distributed as dist
    except ImportError:  # pragma: no cover - torch is part of the environment
        return None
    return dist if dist.is_available() and dist.is_initialized() else None


def EnvInit() -> None:
    """Join the job's process group (gloo, from the launcher's environment) if it has more than
    one process and no group is running yet."""
    global _OWN_GROUP
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if world <= 1 or _dist() is not None:
        return
    import torch.distributed as dist
    os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
    dist.init_process_group("gloo", rank=int(os.environ.get("RANK", "0")), world_size=world)
    _OWN_GROUP = True


def EnvFinalize() -> None:
    """Leave the process group EnvInit started (a group the caller started stays)."""
    global _OWN_GROUP
    d = _dist()
    if d is not None and _OWN_GROUP:
        d.destroy_process_group()
    _OWN_GROUP = False


def EnvFinalizeDummyRanks() -> None:
    """Every rank holds a state here, so no rank is a dummy one: nothing to do."""


class MPIEnvironment:
    """Static queries of the pool of states (one state per process)."""

    @staticmethod
    def GetRank() -> int:
        d = _dist()
        return d.get_rank() if d is not None else 0

    @staticmethod
    def GetSizeWorldComm() -> int:
        d = _dist()
        return d.get_world_size() if d is not None else 1

    @staticmethod
    def IsUsefulRank() -> bool:
        return True

    GetPoolRank = GetRank
    GetPoolSize = GetSizeWorldComm

    @staticmethod
    def GetStateRank() -> int:
        return 0

    @staticmethod
    def GetStateSize() -> int:
        return 1

    @staticmethod
    def GetStateId() -> int:
        return MPIEnvironment.GetRank()

    @staticmethod
    def GetNumStates() -> int:
        return MPIEnvironment.GetSizeWorldComm()

    @staticmethod
    def GetNumRanksPerNode() -> int:
        return int(os.environ.get("LOCAL_WORLD_SIZE", str(MPIEnvironment.GetSizeWorldComm())))

    @staticmethod
    def GetNumNodes() -> int:
        per = max(1, MPIEnvironment.GetNumRanksPerNode())
        return max(1, MPIEnvironment.GetSizeWorldComm() // per)

    @staticmethod
    def Barrier() -> None:
        d = _dist()
        if d is not None:
            d.barrier()

    PoolBarrier = Barrier

    @staticmethod
    def StateBarrier() -> None:
        """A state lives on one process: nothing to wait for."""

    @staticmethod
    def IncoherentSumOverAllStatesOfPool(value: float) -> float:
        """Sum of one double per state over the pool (include/mpi_env.hpp)."""
        d = _dist()
        if d is None:
            return float(value)
        import torch
        t = torch.tensor([float(value)], dtype=torch.float64)
        d.all_reduce(t)
        return float(t.item())

    @staticmethod
    def UpdateStateComm(num_states: int, do_print_info: bool = False) -> None:
        """Only the layout of one state per process exists; any other count is refused."""
        if int(num_states) != MPIEnvironment.GetSizeWorldComm():
            raise ValueError(f"UpdateStateComm: this engine keeps one state per process "
                             f"({MPIEnvironment.GetSizeWorldComm()} states), not {num_states}")
