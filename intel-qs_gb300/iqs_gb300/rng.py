"""The reference's RandomNumberGenerator (include/rng_utils.hpp:46-130, src/rng_utils.cpp:13-225)
over libiqsg's iqsg_rng: a seed and three std::mt19937 streams -- "pool" (seed), "state"
(seed + 1 + state id) and "local" (seed + 1 + number of states + pool rank) -- each with a count
of the numbers drawn or skipped. Each process holds one state, so in a job of P processes
(MPIEnvironment) there are P states and the state id is the pool rank; a single process is a
one-state pool (state id and pool rank 0).

The generator and its distributions live in the C++ library, so the numbers are those of the
reference's standard-library classes. `precision` is the reference's template argument: "DP" for
RandomNumberGenerator<double> (the one its Python module binds), "SP" for <float>; it applies to
this object's own draws. Registers draw in their own precision.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional

import numpy as np

from . import _lib
from ._lib import check, lib

STREAMS = ("pool", "state", "local")
_PREC = {"DP": _lib.COMPLEX_DP, "SP": _lib.COMPLEX_SP}


def _stream(shared: str) -> int:
    if shared not in STREAMS:
        raise ValueError(f"stream must be one of {STREAMS}, not {shared!r}")
    return STREAMS.index(shared)


class RandomNumberGenerator:
    def __init__(self, source: "Optional[RandomNumberGenerator]" = None, *, precision: Optional[str] = None):
        self._h = C.c_void_p()
        if precision is None:
            precision = source.precision if source is not None else "DP"
        if precision not in _PREC:
            raise ValueError(f"precision must be 'DP' or 'SP', not {precision!r}")
        self.precision = precision
        self._p = _PREC[precision]
        if source is not None:  # the copy constructor: same seed, each stream's count skipped
            check(lib.iqsg_rng_clone(source._h, self._p, C.byref(self._h)))
        else:
            check(lib.iqsg_rng_create(C.byref(self._h)))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            lib.iqsg_rng_destroy(h)
            self._h = C.c_void_p()

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    def SetSeedStreamPtrs(self, seed: int) -> None:
        """Seed the three streams; in a pool of several one-state processes (MPIEnvironment) the
        state and local streams differ by state id and pool rank as in the reference."""
        from .environment import MPIEnvironment as E
        check(lib.iqsg_rng_set_seed_pool(self._h, int(seed), E.GetNumStates(), E.GetStateId(), E.GetPoolRank()))

    def _info(self):
        seed = C.c_uint64()
        counts = (C.c_uint64 * 3)()
        check(lib.iqsg_rng_info(self._h, C.byref(seed), counts))
        return seed.value, list(counts)

    def GetSeed(self) -> int:
        return self._info()[0]

    def SkipAhead(self, num_skip: int, shared: str = "local") -> None:
        check(lib.iqsg_rng_skip(self._h, self._p, int(num_skip), _stream(shared)))

    SkipeAhead = SkipAhead  # the name the reference's Python module binds

    def UniformRandomNumbers(self, size: int, a: float = 0.0, b: float = 1.0, shared: str = "local") -> np.ndarray:
        out = np.zeros(int(size))
        check(lib.iqsg_rng_uniform(self._h, self._p, out.ctypes.data_as(_lib._DP), int(size), float(a), float(b),
                                   _stream(shared)))
        return out.astype(np.float32) if self.precision == "SP" else out

    def GetUniformRandomNumbers(self, size: int, a: float, b: float, shared: str) -> list:
        return [float(x) for x in self.UniformRandomNumbers(size, a, b, shared)]

    def GaussianRandomNumbers(self, size: int = 1, shared: str = "local") -> np.ndarray:
        out = np.zeros(int(size))
        check(lib.iqsg_rng_gaussian(self._h, self._p, out.ctypes.data_as(_lib._DP), int(size), _stream(shared)))
        return out.astype(np.float32) if self.precision == "SP" else out

    def RandomIntegersInRange(self, size: int, a: int, b: int, shared: str = "local") -> np.ndarray:
        out = np.zeros(int(size), dtype=np.int32)
        check(lib.iqsg_rng_integers(self._h, self._p, out.ctypes.data_as(C.POINTER(C.c_int)), int(size), int(a),
                                    int(b), _stream(shared)))
        return out

    def GetNumGeneratedOrSkippedPoolNumbers(self) -> int:
        return self._info()[1][0]

    def GetNumGeneratedOrSkippedStateNumbers(self) -> int:
        return self._info()[1][1]

    def GetNumGeneratedOrSkippedLocalNumbers(self) -> int:
        return self._info()[1][2]

    def __repr__(self) -> str:
        return f"<RandomNumberGenerator {self.precision} seed={self.GetSeed()}>"
