"""The reference's RandomNumberGenerator (include/rng_utils.hpp, src/rng_utils.cpp:20-160) as
far as register initialisation needs it: a seed and three streams -- "pool" (std::mt19937
seeded with seed), "state" (seed + 1 + state id) and "local" (seed + 1 + number of states +
pool rank) -- each with a count of the numbers drawn or skipped. One process is one state of a
one-state pool here, so the state id and pool rank are 0 and the number of states is 1.

The numbers themselves are drawn where they are used (iqsg_init_uniform_random regenerates a
stream from its seed and skips the counted numbers), so skipping is only a count.
"""
from __future__ import annotations

STREAMS = ("pool", "state", "local")


class RandomNumberGenerator:
    def __init__(self, source: "RandomNumberGenerator | None" = None):
        self._seed = 0
        self._count = {s: 0 for s in STREAMS}
        if source is not None:  # the copy constructor: same seed, same positions
            self._seed = source._seed
            self._count = dict(source._count)

    def SetSeedStreamPtrs(self, seed: int) -> None:
        self._seed = int(seed)
        self._count = {s: 0 for s in STREAMS}

    def GetSeed(self) -> int:
        return self._seed

    def SkipAhead(self, num_skip: int, shared: str) -> None:
        if shared not in STREAMS:
            raise ValueError(f"stream must be one of {STREAMS}, not {shared!r}")
        self._count[shared] += int(num_skip)

    def GetNumGeneratedOrSkippedPoolNumbers(self) -> int:
        return self._count["pool"]

    def GetNumGeneratedOrSkippedStateNumbers(self) -> int:
        return self._count["state"]

    def GetNumGeneratedOrSkippedLocalNumbers(self) -> int:
        return self._count["local"]

    def stream_seed(self, shared: str) -> int:
        """Seed of the std::mt19937 behind a stream (src/rng_utils.cpp:64-78)."""
        return {"pool": self._seed, "state": self._seed + 1, "local": self._seed + 2}[shared]
