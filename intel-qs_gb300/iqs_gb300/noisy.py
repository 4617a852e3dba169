"""NoisyQureg (include/NoisyQureg.hpp of intel/intel-qs): a register that adds a Pauli-twirl noise
gate for the idle time of each qubit before every logical gate.

Every qubit keeps the time since its last gate. Before a 1-qubit gate on q (2-qubit gate on q1, q2)
the noise gate for q's idle time is applied, every qubit's idle time grows by the gate duration,
and q's is reset to zero. Noise angles come from the class's own std::default_random_engine
(seeded by the constructor) through a std::normal_distribution of the base type, drawn in
libiqsg. Times are kept in the base type (float for ComplexSP) as the reference keeps them.
Gates other than the ones listed below (ApplyPauliX, Apply2QubitGate, ...) run without noise, as
they do in the reference, whose gate methods are not virtual.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import check, lib
from .qureg import QubitRegister


class NoisyQureg(QubitRegister):
    def __init__(self, num_qubits: int, RNG_seed: int = 12345, T1: float = 2000.0, T2: float = 1000.0, *,
                 precision: str = "DP", math: str = "native"):
        super().__init__(num_qubits, "", 0, precision=precision, math=math)
        self._ft = np.float64 if precision == "DP" else np.float32
        self.T_1 = self._ft(T1)
        self.T_2 = self._ft(T2)
        self.time_one_qubit_experimental_gate = self._ft(1.0)
        self.time_two_qubit_experimental_gate = self._ft(1.0)
        self.time_from_last_gate = np.zeros(num_qubits, dtype=self._ft)
        self._count_matrix = np.zeros((num_qubits, num_qubits), dtype=np.int64)
        self._one_count = 0
        self._two_count = 0
        self._busy = False
        self._engine = C.c_void_p()
        check(lib.iqsg_noise_engine_create(int(RNG_seed) & 0xFFFFFFFF, C.byref(self._engine)))

    def __del__(self):
        e = getattr(self, "_engine", None)
        if e is not None and e.value:
            lib.iqsg_noise_engine_destroy(e)
            self._engine = C.c_void_p()
        super().__del__()

    # ---- state and settings ----------------------------------------------------------
    def Initialize(self, style: str = "", base_index: int = 0) -> None:
        if hasattr(self, "_engine"):
            self._one_count = 0
            self._two_count = 0
            self.ResetTimeForAllQubits()
        super().Initialize(style, base_index)

    def ResetTimeForAllQubits(self) -> None:
        self.time_from_last_gate[:] = 0

    def ApplyNoiseGatesOnAllQubits(self) -> None:
        """Noise for each qubit's idle time since its last gate, then all idle times reset."""
        for q in range(self.NumQubits()):
            self.NoiseGate(q)
        self.ResetTimeForAllQubits()

    def SetDecoherenceTime(self, T1: float, T2: float) -> None:
        self.T_1, self.T_2 = self._ft(T1), self._ft(T2)

    def SetGateDurations(self, Ts: float, Td: float) -> None:
        self.time_one_qubit_experimental_gate = self._ft(Ts)
        self.time_two_qubit_experimental_gate = self._ft(Td)

    # ---- counts -------------------------------------------------------------------------
    def GetOneQubitExperimentalGateCount(self) -> int:
        return self._one_count

    def GetTwoQubitExperimentalGateCount(self) -> int:
        return self._two_count

    def GetTotalExperimentalGateCount(self) -> int:
        return self._one_count + self._two_count

    def GetExperimentalGateCount(self, q1: int, q2=None):
        """Row q1 of the gate-count matrix, or its entry (q1, q2)."""
        if q2 is None:
            return [int(x) for x in self._count_matrix[q1]]
        return int(self._count_matrix[q1, q2])

    # ---- noise ----------------------------------------------------------------------------
    def NoiseGate(self, qubit: int) -> None:
        t = self.time_from_last_gate[qubit]
        if t == 0:
            return
        g = np.zeros(3)
        check(lib.iqsg_noise_engine_gaussian(self._engine, self._prec, g.ctypes.data_as(_lib._DP), 3))
        m = np.zeros(8)
        check(lib.iqsg_noise_gate_matrix(self._prec, float(self.T_1), float(self.T_2), float(t),
                                         g.ctypes.data_as(_lib._DP), m.ctypes.data_as(_lib._DP)))
        busy, self._busy = self._busy, True
        try:
            QubitRegister.Apply1QubitGate(self, qubit, m.view(np.complex128).reshape(2, 2))
        finally:
            self._busy = busy

    def AddNoiseOneQubitGate(self, qubit: int) -> None:
        self.NoiseGate(qubit)
        self.time_from_last_gate += self.time_one_qubit_experimental_gate
        self.time_from_last_gate[qubit] = 0
        self._one_count += 1
        self._count_matrix[qubit, qubit] += 1

    def AddNoiseTwoQubitGate(self, q1: int, q2: int) -> None:
        self.NoiseGate(q1)
        self.NoiseGate(q2)
        self.time_from_last_gate += self.time_two_qubit_experimental_gate
        self.time_from_last_gate[q1] = 0
        self.time_from_last_gate[q2] = 0
        self._two_count += 1
        self._count_matrix[q1, q2] += 1
        self._count_matrix[q2, q1] += 1

    def _noisy(self, add, base, *args, **kw):
        # Gates that the listed gates issue internally run without further noise.
        if self._busy:
            return base(self, *args, **kw)
        add()
        self._busy = True
        try:
            return base(self, *args, **kw)
        finally:
            self._busy = False

    # ---- gates with noise (include/NoisyQureg.hpp:449-505) --------------------------------
    def Apply1QubitGate(self, qubit: int, m, *args, **kw) -> None:
        self._noisy(lambda: self.AddNoiseOneQubitGate(qubit), QubitRegister.Apply1QubitGate, qubit, m, *args, **kw)

    def ApplyHadamard(self, qubit: int) -> None:
        self._noisy(lambda: self.AddNoiseOneQubitGate(qubit), QubitRegister.ApplyHadamard, qubit)

    def ApplyRotationX(self, qubit: int, theta: float) -> None:
        self._noisy(lambda: self.AddNoiseOneQubitGate(qubit), QubitRegister.ApplyRotationX, qubit, theta)

    def ApplyRotationY(self, qubit: int, theta: float) -> None:
        self._noisy(lambda: self.AddNoiseOneQubitGate(qubit), QubitRegister.ApplyRotationY, qubit, theta)

    def ApplyRotationZ(self, qubit: int, theta: float) -> None:
        self._noisy(lambda: self.AddNoiseOneQubitGate(qubit), QubitRegister.ApplyRotationZ, qubit, theta)

    def ApplyCPauliX(self, control: int, target: int) -> None:
        self._noisy(lambda: self.AddNoiseTwoQubitGate(control, target), QubitRegister.ApplyCPauliX, control, target)

    def ApplyControlled1QubitGate(self, control: int, target: int, m, *args, **kw) -> None:
        self._noisy(lambda: self.AddNoiseTwoQubitGate(control, target), QubitRegister.ApplyControlled1QubitGate,
                    control, target, m, *args, **kw)


def _plain(name: str):
    def f(self, *args, **kw):
        busy, self._busy = self._busy, True
        try:
            return getattr(QubitRegister, name)(self, *args, **kw)
        finally:
            self._busy = busy
    f.__name__ = name
    f.__doc__ = f"QubitRegister.{name} without noise (the reference does not override it)."
    return f


# Gates without noise that the base class builds from the ones with noise.
for _name in ("ApplyPauliX", "ApplyPauliY", "ApplyPauliZ", "ApplyPauliSqrtX", "ApplyPauliSqrtY", "ApplyPauliSqrtZ",
              "ApplyS", "ApplyT", "ApplyRotationXY", "ApplyCRotationX", "ApplyCRotationY", "ApplyCRotationZ",
              "ApplyCPauliY", "ApplyCPauliZ", "ApplyCPauliSqrtZ", "ApplyCHadamard", "ApplyCPhaseRotation",
              "ApplyToffoli", "ApplyNoiseGate", "ApplyChannel"):
    if hasattr(QubitRegister, _name):
        setattr(NoisyQureg, _name, _plain(_name))
del _name


class QubitRegisterMetric(QubitRegister):
    """QubitRegisterMetric (include/QubitRegisterMetric.hpp): the gates below also count 1- and
    2-qubit gates and track a per-qubit depth (a 2-qubit gate puts both qubits at one more than
    the deeper of the two). Other gates are not counted, as in the reference."""

    def __init__(self, num_qubits: int, *, precision: str = "DP", math: str = "native"):
        super().__init__(num_qubits, "", 0, precision=precision, math=math)
        self._total = self._one = self._two = 0
        self._depth = [0] * num_qubits
        self._inside = False

    def GetTotalQubitGateCount(self) -> int:
        return self._total

    def GetOneQubitGateCount(self) -> int:
        return self._one

    def GetTwoQubitGateCount(self) -> int:
        return self._two

    def GetParallelDepth(self) -> int:
        return max(self._depth) if self._depth else 0

    def _count(self, base, qs, *args):
        if self._inside:  # a counted gate built from another counted one counts once
            return base(self, *args)
        self._inside = True
        try:
            base(self, *args)
        finally:
            self._inside = False
        self._total += 1
        if len(qs) == 1:
            self._one += 1
            self._depth[qs[0]] += 1
        else:
            self._two += 1
            d = max(self._depth[qs[0]], self._depth[qs[1]]) + 1
            self._depth[qs[0]] = self._depth[qs[1]] = d

    def ApplyHadamard(self, q: int) -> None:
        self._count(QubitRegister.ApplyHadamard, (q,), q)

    def ApplyRotationX(self, q: int, theta: float) -> None:
        self._count(QubitRegister.ApplyRotationX, (q,), q, theta)

    def ApplyRotationY(self, q: int, theta: float) -> None:
        self._count(QubitRegister.ApplyRotationY, (q,), q, theta)

    def ApplyRotationZ(self, q: int, theta: float) -> None:
        self._count(QubitRegister.ApplyRotationZ, (q,), q, theta)

    def ApplyCPauliX(self, q1: int, q2: int) -> None:
        self._count(QubitRegister.ApplyCPauliX, (q1, q2), q1, q2)

    def ApplyControlled1QubitGate(self, q1: int, q2: int, m, *args, **kw) -> None:
        self._count(lambda s, *a: QubitRegister.ApplyControlled1QubitGate(s, *a, **kw), (q1, q2), q1, q2, m, *args)
