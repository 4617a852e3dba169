"""QubitRegister: the iqs::QubitRegister<Type> API over libiqsg (GPU state in HBM).

Method names, argument order and meaning follow the reference class (include/qureg.hpp:
127-417) and its Python binding (pybind11/intelqs_py.cpp:173-352). Qubit arguments are
program qubits; this class keeps the Permutation and translates them to data positions
before each call into libiqsg, as the reference's helpers do. Where the reference asserts
on bad input, these methods raise ValueError.
"""
from __future__ import annotations

import cmath
import ctypes as C
import math
from typing import Optional, Sequence

import numpy as np

from . import _lib
from ._lib import check, dptr, lib, uptr
from .permutation import GateCounter, Permutation, check_distinct

_PREC = {"DP": _lib.COMPLEX_DP, "SP": _lib.COMPLEX_SP, "ComplexDP": _lib.COMPLEX_DP, "ComplexSP": _lib.COMPLEX_SP}
_MATH = {"native": _lib.MATH_NATIVE, "emulated": _lib.MATH_EMULATED}


def _m2(m) -> np.ndarray:
    a = np.ascontiguousarray(np.asarray(m, dtype=np.complex128))
    if a.ndim != 2 or a.shape != (2, 2):
        raise ValueError(f"expected a 2x2 matrix, got shape {a.shape}")
    return a.reshape(-1).view(np.float64).copy()


def _op(kind: int, t0: int = 0, t1: int = 0, m=None, ctrl=(), mask: int = 0, value: int = 0) -> "_lib.Op":
    op = _lib.Op()
    op.kind, op.t0, op.t1 = kind, t0, t1
    op.nctrl = len(ctrl)
    for k, c in enumerate(ctrl):
        op.ctrl[k] = c
    op.mask, op.value = mask, value
    if m is not None:
        C.memmove(op.m, m.ctypes.data, m.nbytes)
    return op


def _m4(m) -> np.ndarray:
    a = np.ascontiguousarray(np.asarray(m, dtype=np.complex128))
    if a.ndim != 2 or a.shape != (4, 4):
        raise ValueError(f"expected a 4x4 matrix, got shape {a.shape}")
    return a.reshape(-1).view(np.float64).copy()


class QubitRegister:
    """State of ``num_qubits`` qubits held in GPU memory.

    QubitRegister()                                  -> 1 qubit in |0>
    QubitRegister(other)                             -> deep copy (device to device)
    QubitRegister(n, style="", base_index=0, tmp_spacesize=0, precision="DP")
        style "base": |base_index>, "++++": uniform superposition, "": all zeros.

    ``precision`` selects ComplexDP ("DP") or ComplexSP ("SP") storage; ``math`` selects
    native FP64 or emulated-FP64 arithmetic for ComplexDP gates; ``stream`` is an optional
    cudaStream_t (int) to queue the register's work on.
    """

    def __init__(self, num_qubits=None, style: str = "", base_index: int = 0, tmp_spacesize: int = 0, *,
                 precision: str = "DP", math: str = "native", stream: Optional[int] = None):
        self._h = C.c_void_p()
        if isinstance(num_qubits, QubitRegister):
            src = num_qubits
            src._flush()
            check(lib.iqsg_clone(src._h, C.byref(self._h)))
            self._n, self._prec = src._n, src._prec
            self.qubit_permutation = src.qubit_permutation.copy()
            self._init_flags()
            self._math = src._math
            return
        if num_qubits is None:
            num_qubits, style, base_index = 1, "base", 0
        if precision not in _PREC:
            raise ValueError(f"precision must be 'DP' or 'SP', not {precision!r}")
        self._n = int(num_qubits)
        self._prec = _PREC[precision]
        check(lib.iqsg_create(self._n, self._prec, C.c_void_p(stream or 0), C.byref(self._h)))
        self.qubit_permutation = Permutation(self._n)
        self._init_flags()
        self.SetMath(math)
        self.Initialize(style, base_index)

    @classmethod
    def from_device(cls, num_qubits: int, device_ptr: int, *, precision: str = "DP", stream: Optional[int] = None,
                    math: str = "native") -> "QubitRegister":
        """Wrap caller-owned device memory (the imported-state constructor,
        src/qureg_init.cpp:193-200). The memory is not freed by this object."""
        self = cls.__new__(cls)
        self._h = C.c_void_p()
        self._n = int(num_qubits)
        self._prec = _PREC[precision]
        check(lib.iqsg_create_from_device(self._n, self._prec, C.c_void_p(device_ptr), C.c_void_p(stream or 0),
                                          C.byref(self._h)))
        self.qubit_permutation = Permutation(self._n)
        self._init_flags()
        self.SetMath(math)
        return self

    def _init_flags(self):
        self._rng = None
        self.gate_counter: Optional[GateCounter] = None
        self._queue = []
        self.fusion = False
        self.log2llc = 20
        self.specialize = False
        self.specialize2 = False
        self._math = _lib.MATH_NATIVE

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            lib.iqsg_destroy(h)
            self._h = C.c_void_p()

    # ---- information ---------------------------------------------------------------
    def NumQubits(self) -> int:
        return self._n

    def GlobalSize(self) -> int:
        return 1 << self._n

    def LocalSize(self) -> int:
        return 1 << self._n

    def size(self) -> int:
        return 1 << self._n

    @property
    def num_qubits(self) -> int:
        return self._n

    @property
    def precision(self) -> str:
        return "DP" if self._prec == _lib.COMPLEX_DP else "SP"

    @property
    def dtype(self):
        return np.complex128 if self._prec == _lib.COMPLEX_DP else np.complex64

    def SetMath(self, math: str) -> None:
        """'native' (IEEE FP64) or 'emulated' (double-float) arithmetic for ComplexDP gates."""
        if math not in _MATH:
            raise ValueError(f"math must be 'native' or 'emulated', not {math!r}")
        self._math = _MATH[math]
        check(lib.iqsg_set_math(self._h, self._math))

    def RawState(self) -> int:
        """Device address of amplitude 0 (the reference returns its host array). The
        address can change after PermuteQubits."""
        p = C.c_void_p()
        check(lib.iqsg_info(self._h, None, None, C.byref(p)))
        return p.value or 0

    @property
    def __cuda_array_interface__(self):
        return {"shape": (1 << self._n,), "typestr": "<c16" if self._prec == _lib.COMPLEX_DP else "<c8",
                "data": (self.RawState(), False), "version": 3, "strides": None}

    def synchronize(self) -> None:
        check(lib.iqsg_synchronize(self._h))

    def _bt(self, x: float) -> float:
        """The value as the reference's BaseType would hold it (float for ComplexSP)."""
        return float(np.float32(x)) if self._prec == _lib.COMPLEX_SP else float(x)

    # ---- state initialisation / access -----------------------------------------------
    def Initialize(self, style: str = "", base_index: int = 0) -> None:
        """src/qureg_init.cpp:225-359: "base", "++++", "" (all zero) and "rand" (needs SetRngPtr)."""
        if style == "base":
            if not 0 <= base_index < self.GlobalSize():
                raise ValueError(f"base_index {base_index} out of range")
            check(lib.iqsg_init_basis(self._h, self.qubit_permutation.program2data_(int(base_index))))
        elif style == "++++":
            check(lib.iqsg_fill(self._h, self._bt(1.0 / math.sqrt(self.GlobalSize())), 0.0))
        elif style == "":
            check(lib.iqsg_fill(self._h, 0.0, 0.0))
        elif style == "rand":
            # src/qureg_init.cpp:253-330: real and imaginary parts uniform in [-1, 1) from the
            # register's RNG ("pool" stream for base_index 0, "local" for base_index = number of
            # states = 1), the stream advanced by 2 * 2^n, then the state normalised.
            rng = self._rng
            if rng is None:
                raise ValueError("Initialize('rand'): set a RandomNumberGenerator with SetRngPtr first")
            if rng.GetSeed() == 0:
                raise ValueError("Initialize('rand'): the RandomNumberGenerator needs a nonzero seed")
            if base_index not in (0, 1):
                raise ValueError("Initialize('rand'): base_index must be 0 (pool stream) or 1 (local stream)")
            self._flush()
            check(lib.iqsg_init_random(self._h, rng.handle, 0 if base_index == 0 else 2))
            self.Normalize()
        else:
            raise ValueError(f"unknown initialisation style {style!r}")

    # ---- random number generator (include/qureg.hpp:375-379) ----------------------------
    def SetRngPtr(self, rng) -> None:
        self._rng = rng

    def GetRngPtr(self):
        return self._rng

    def ResetRngPtr(self) -> None:
        self._rng = None

    def SetSeedRngPtr(self, seed: int) -> None:
        if self._rng is None:
            raise ValueError("SetSeedRngPtr: no RandomNumberGenerator set")
        self._rng.SetSeedStreamPtrs(seed)

    # ---- noise (src/qureg_noisysimul.cpp, src/qureg_apply_channel.cpp) --------------------
    def SetNoiseTimescales(self, T1: float, T2: float) -> None:
        """Dissipation time T1 and decoherence time T2 (T2 >= T1/2); T_phi = 1/(1/T2 - 1/(2 T1))."""
        T1, T2 = self._bt(T1), self._bt(T2)
        if not T2 >= T1 / 2.0:
            raise ValueError(f"SetNoiseTimescales: T2 = {T2} must be at least T1/2 = {T1 / 2.0}")
        self._T1, self._T2 = T1, T2
        with np.errstate(divide="ignore"):
            self._Tphi = self._bt(1.0 / (1.0 / T2 - 1.0 / (2.0 * T1))) if T2 != T1 / 2.0 else float("inf")

    def GetT1(self) -> float:
        return getattr(self, "_T1", 0.0)

    def GetT2(self) -> float:
        return getattr(self, "_T2", 0.0)

    def GetTphi(self) -> float:
        return getattr(self, "_Tphi", 0.0)

    def ApplyNoiseGate(self, qubit: int, duration: float) -> None:
        """Pauli-twirl noise for `duration` on `qubit` (src/qureg_noisysimul.cpp:33-85): three
        Gaussian angles from the RNG's "state" stream, one 1-qubit gate."""
        if self._rng is None:
            raise ValueError("ApplyNoiseGate: set a RandomNumberGenerator with SetRngPtr first")
        if not hasattr(self, "_T1"):
            raise ValueError("ApplyNoiseGate: call SetNoiseTimescales first")
        duration = self._bt(duration)
        if duration == 0:
            return
        m = np.zeros(8)
        check(lib.iqsg_noise_gate_draw(self._rng.handle, self._prec, self._T1, self._T2, duration,
                                       m.ctypes.data_as(_lib._DP)))
        QubitRegister.Apply1QubitGate(self, qubit, m.view(np.complex128).reshape(2, 2))

    def ApplyChannel(self, *args) -> None:
        """ApplyChannel(qubit, chi) with a 4x4 chi matrix, or ApplyChannel(qubit1, qubit2, chi)
        with a 16x16 one (src/qureg_apply_channel.cpp:17-106): one eigenvector of chi, drawn with
        probability |E_k| / sum |E| from the RNG's "state" stream, applied as a gate; a negative
        eigenvalue flips GetOverallSignOfChannels()."""
        if len(args) == 2:
            qubits, chi, M = args[:1], args[1], 4
        elif len(args) == 3:
            qubits, chi, M = args[:2], args[2], 16
        else:
            raise TypeError("ApplyChannel(qubit, chi) or ApplyChannel(qubit1, qubit2, chi)")
        if getattr(chi, "M", None) != M:
            raise ValueError(f"ApplyChannel on {len(qubits)} qubit(s) needs a {M}x{M} chi matrix")
        if chi.precision != self.precision:
            raise ValueError(f"ApplyChannel: chi matrix is {chi.precision}, the register {self.precision}")
        if self._rng is None:
            raise ValueError("ApplyChannel: set a RandomNumberGenerator with SetRngPtr first")
        ev, cum, vf = chi._arrays()
        gate = np.zeros(2 * (2 if M == 4 else 4) ** 2)
        k, neg = C.c_uint(), C.c_int()
        check(lib.iqsg_channel_gate(self._rng.handle, self._prec, M, ev.ctypes.data_as(_lib._DP),
                                    cum.ctypes.data_as(_lib._DP), vf.ctypes.data_as(_lib._DP),
                                    gate.ctypes.data_as(_lib._DP), C.byref(k), C.byref(neg)))
        if neg.value:
            self._overall_sign = -self.GetOverallSignOfChannels()
        g = gate.view(np.complex128)
        if M == 4:
            QubitRegister.Apply1QubitGate(self, qubits[0], g.reshape(2, 2))
        else:
            QubitRegister.Apply2QubitGate(self, qubits[0], qubits[1], g.reshape(4, 4))

    def GetOverallSignOfChannels(self) -> float:
        return getattr(self, "_overall_sign", 1.0)

    def InitializationWithSameAmplitudeEverywhere(self, amplitude: complex) -> None:
        a = complex(amplitude)
        check(lib.iqsg_fill(self._h, a.real, a.imag))

    def GetStateVector(self, out: Optional[np.ndarray] = None) -> np.ndarray:
        """All amplitudes in data order, copied to host memory: a new array, or ``out``
        (contiguous, this register's dtype; pinned memory makes the copy faster)."""
        if out is None:
            out = np.empty(self.GlobalSize(), dtype=self.dtype)
        elif out.dtype != self.dtype or out.shape != (self.GlobalSize(),) or not out.flags.c_contiguous:
            raise ValueError("GetStateVector: out must be a contiguous array of this register's size and dtype")
        check(lib.iqsg_download(self._h, out.ctypes.data_as(C.c_void_p), 0, out.size))
        return out

    def SetStateVector(self, amps) -> None:
        """Overwrite all amplitudes (data order) from a host array."""
        a = np.ascontiguousarray(np.asarray(amps, dtype=self.dtype))
        if a.shape != (self.GlobalSize(),):
            raise ValueError(f"expected {self.GlobalSize()} amplitudes, got shape {a.shape}")
        check(lib.iqsg_upload(self._h, a.ctypes.data_as(C.c_void_p), 0, a.size))

    def SetStateVectorAsync(self, amps: np.ndarray) -> None:
        """Queue the upload of all amplitudes from a contiguous host array of this register's
        dtype (pinned memory makes it asynchronous); it runs in order with the register's
        gates. Keep the array alive and unchanged until synchronize()."""
        self._flush()
        if amps.dtype != self.dtype or amps.shape != (self.GlobalSize(),) or not amps.flags.c_contiguous:
            raise ValueError("SetStateVectorAsync: amps must be a contiguous array of this register's size and dtype")
        check(lib.iqsg_upload_async(self._h, amps.ctypes.data_as(C.c_void_p), 0, amps.size))

    def GetStateVectorAsync(self, out: np.ndarray) -> np.ndarray:
        """Queue the download of all amplitudes into `out` (contiguous, this register's dtype);
        the data is there after synchronize()."""
        self._flush()
        if out.dtype != self.dtype or out.shape != (self.GlobalSize(),) or not out.flags.c_contiguous:
            raise ValueError("GetStateVectorAsync: out must be a contiguous array of this register's size and dtype")
        check(lib.iqsg_download_async(self._h, out.ctypes.data_as(C.c_void_p), 0, out.size))
        return out

    def __array__(self, dtype=None, copy=None):
        a = self.GetStateVector()
        return a if dtype is None else a.astype(dtype)

    def __getitem__(self, index: int) -> complex:
        """Amplitude at a data (local) index, like the reference's operator[]."""
        if not 0 <= index < self.LocalSize():
            raise IndexError(index)
        out = (C.c_double * 2)()
        check(lib.iqsg_get_amplitude(self._h, int(index), out))
        return complex(out[0], out[1])

    def __setitem__(self, index: int, value: complex) -> None:
        if not 0 <= index < self.LocalSize():
            raise IndexError(index)
        v = complex(value)
        check(lib.iqsg_set_amplitude(self._h, int(index), v.real, v.imag))

    def GetGlobalAmplitude(self, index: int) -> complex:
        """src/qureg_utils.cpp:78-99 (index in program-qubit order)."""
        if not 0 <= index < self.GlobalSize():
            raise ValueError(f"index {index} out of range")
        return self[self.qubit_permutation.program2data_(int(index))]

    def SetGlobalAmplitude(self, index: int, value: complex) -> None:
        """src/qureg_utils.cpp:104-121."""
        if not 0 <= index < self.GlobalSize():
            raise ValueError(f"index {index} out of range")
        self[self.qubit_permutation.program2data_(int(index))] = value

    # ---- state statistics and output formats --------------------------------------------
    def GoogleStats(self) -> list:
        """[entropy, average self-information, scaled moments m2..m10] in one pass on the GPU
        (src/qureg_utils.cpp:349-450)."""
        self._flush()
        out = (C.c_double * 11)()
        check(lib.iqsg_state_stats(self._h, out))
        return [float(x) for x in out]

    def Entropy(self) -> float:
        """-sum p log2 p over the amplitudes (src/qureg_utils.cpp:303-346)."""
        return self.GoogleStats()[0]

    def _norms(self, a: np.ndarray) -> np.ndarray:
        if self._prec == _lib.COMPLEX_SP:  # std::norm in float
            return (a.real * a.real + a.imag * a.imag).astype(np.float32)
        return a.real * a.real + a.imag * a.imag

    def Print(self, x: str, qubits=()) -> None:
        """Print the qubit map and every amplitude with its program-order basis string and
        probability, in the reference's format (src/qureg_utils.cpp:461-563; `qubits` is
        unused there too). Copies the state to the host."""
        a = self.GetStateVector()
        p = self._norms(a)
        perm = self.qubit_permutation
        lines = [f"qubit permutation: {perm.GetMapStr()}", f"{x}=["]
        for i in range(a.size):
            lines.append("\t%-13.8f + i * %-13.8f   %% |%s> p=%f" % (a[i].real, a[i].imag, perm.data2program(i), p[i]))
        cum = np.cumsum(p)[-1] if a.size else 0.0  # accumulated in the register's precision
        lines.append("]; %% cumulative probability = %f" % float(cum))
        print("\n".join(lines), flush=True)

    def ExportAmplitudes(self, ofname: str) -> None:
        """Append the amplitudes as JSON members "bits" : [re, im, p] to ofname, in the
        reference's format (src/qureg_utils.cpp:566-657)."""
        a = self.GetStateVector()
        p = self._norms(a)
        perm = self.qubit_permutation
        body = "".join("\t\t\"%s\" : [%-13.8f, %-13.8f, %f],\n" % (perm.data2program(i), a[i].real, a[i].imag, p[i])
                       for i in range(a.size))
        body = body[:-2] + "\n"  # no comma after the last member
        with open(ofname, "a") as f:
            f.write("\t\"amplitudes\" :\n\t{\n" + body + "\t}\n")

    def dumpbin(self, fn: str) -> None:
        """Write the raw amplitudes (data order, the register's complex type) to fn, as the
        reference's MPI build does on one rank (src/qureg_utils.cpp:661-689)."""
        import time
        t0 = time.perf_counter()
        a = self.GetStateVector()
        a.tofile(fn)
        dt = time.perf_counter() - t0
        print("Dumping state to %s took %f sec (%f MB/s)" % (fn, dt, a.nbytes / max(dt, 1e-12) / 1e6), flush=True)

    # ---- statistics ---------------------------------------------------------------------
    def EnableStatistics(self) -> None:
        self.gate_counter = GateCounter(self._n)

    def DisableStatistics(self) -> None:
        self.gate_counter = None

    def ResetStatistics(self) -> None:
        if self.gate_counter:
            self.gate_counter = GateCounter(self._n)

    def GetStatistics(self) -> Optional[str]:
        return self.gate_counter.Breakdown() if self.gate_counter else None

    def _count1(self, q):
        if self.gate_counter is not None:
            self.gate_counter.OneQubitIncrement(q)

    def _count2(self, q0, q1):
        if self.gate_counter is not None:
            self.gate_counter.TwoQubitIncrement(q0, q1)

    # ---- fusion / specialisation toggles ----------------------------------------------------
    def TurnOnFusion(self, log2llc: int = 20) -> None:
        """Queue gates and apply them in fused sweeps (iqsg_apply_ops): each pass over the
        state applies several gates in registers. The reference buffers gates below
        position log2llc and replays them block by block (src/qureg_fusion.cpp:12-94);
        here every gate is queued, whatever its position, and the queue is applied before
        anything reads or reorders the state. Results equal the unfused ones."""
        self.fusion = True
        self.log2llc = int(log2llc)

    def TurnOffFusion(self) -> None:
        self.ApplyFusedGates()
        self.fusion = False

    def IsFusionEnabled(self) -> bool:
        return self.fusion

    def ApplyFusedGates(self) -> int:
        """Apply the queued gates; returns the number of passes over the state it took."""
        if not self._queue:
            return 0
        arr = (_lib.Op * len(self._queue))(*self._queue)
        self._queue = []
        sweeps = C.c_uint()
        check(lib.iqsg_apply_ops(self._h, arr, len(arr), C.byref(sweeps)))
        return sweeps.value

    _flush = ApplyFusedGates

    def PlanFusedGates(self) -> dict:
        """The passes ApplyFusedGates would run for the queued gates, without running them
        (see plan_ops)."""
        return plan_ops(self._n, self._queue, precision=self.precision,
                        math="emulated" if self._math == _lib.MATH_EMULATED else "native",
                        width=getattr(self, "_width", 0))

    def SetSweepWidth(self, kmax: int) -> None:
        """Largest number of target qubits one fused pass holds in registers (1..4, 0 =
        default for the precision)."""
        self._flush()
        check(lib.iqsg_set_sweep_width(self._h, int(kmax)))
        self._width = int(kmax)

    def SetNativeShare(self, sixteenths: int) -> None:
        """Emulated ComplexDP fused sweeps: let sixteenths/16 of the warps use native FP64 (the
        FP64 pipe runs alongside the FP32 pipes); results change only by rounding."""
        self._flush()
        check(lib.iqsg_set_option(self._h, _lib.OPT_NATIVE_SHARE, int(sixteenths)))

    def SetDoubleFloatStorage(self, on: bool) -> None:
        """Emulated ComplexDP gate streams of 3+ sweeps: keep the state as double-float pairs
        between sweeps (default on); off, every sweep reads and writes FP64. Rounding only."""
        self._flush()
        check(lib.iqsg_set_option(self._h, _lib.OPT_DF_STORAGE, 1 if on else 0))

    def counters(self) -> dict:
        """Double-float storage runs started by fused gate streams and the kernels they launched."""
        c = (C.c_uint64 * 2)()
        check(lib.iqsg_counters(self._h, c))
        return {"df_runs": int(c[0]), "df_launches": int(c[1])}

    def SetTileQubits(self, k: int) -> None:
        """Run fused gate streams as shared-memory tile passes spanning k positions (0 = off,
        register sweeps only); a tuning choice that changes results only by rounding (gates
        on disjoint qubits may be applied in a different order)."""
        self._flush()
        check(lib.iqsg_set_option(self._h, _lib.OPT_TILE_QUBITS, int(k)))

    def SetSweepPipeline(self, on: bool) -> None:
        """Stream fused passes through shared memory with bulk async copies (registers of 16+
        qubits); a tuning choice that never changes results."""
        self._flush()
        check(lib.iqsg_set_option(self._h, _lib.OPT_SWEEP_PIPELINE, 1 if on else 0))

    def _enqueue(self, op) -> None:
        self._queue.append(op)
        if len(self._queue) >= 4096:
            self._flush()

    def TurnOnSpecialize(self) -> None:
        self.specialize = True

    def TurnOffSpecialize(self) -> None:
        self.specialize = False

    def TurnOnSpecializeV2(self) -> None:
        self.specialize2 = True

    def TurnOffSpecializeV2(self) -> None:
        self.specialize2 = False

    # ---- position helpers -----------------------------------------------------------------
    def _pos(self, q: int, what: str) -> int:
        if not 0 <= q < self._n:
            raise ValueError(f"{what}: qubit {q} out of range for {self._n} qubits")
        return self.qubit_permutation.map[q]

    # ---- generic gates ------------------------------------------------------------------------
    def Apply1QubitGate(self, qubit: int, m, spec=None, angle: float = 0.0) -> None:
        """src/qureg_apply1qubitgate.cpp:234-265."""
        m8 = _m2(m)
        p = self._pos(qubit, "Apply1QubitGate")
        self._count1(qubit)
        if self.fusion:
            self._enqueue(_op(_lib.OP_1Q, p, 0, m8))
        else:
            check(lib.iqsg_apply_1q(self._h, p, dptr(m8)))

    def ApplyControlled1QubitGate(self, control: int, target: int, m, spec=None, angle: float = 0.0) -> None:
        """src/qureg_applyctrl1qubitgate.cpp:414-444."""
        m8 = _m2(m)
        pc, pt = self._pos(control, "ApplyControlled1QubitGate"), self._pos(target, "ApplyControlled1QubitGate")
        if control == target:
            raise ValueError("ApplyControlled1QubitGate: control and target coincide")
        self._count2(control, target)
        if self.fusion:
            self._enqueue(_op(_lib.OP_CTRL, pt, 0, m8, ctrl=(pc,)))
        else:
            check(lib.iqsg_apply_controlled_1q(self._h, pc, pt, dptr(m8)))

    def Apply2QubitGate(self, qubit_high: int, qubit_low: int, m) -> None:
        """src/qureg_apply2qubitgate.cpp:14-73."""
        m32 = _m4(m)
        ph, pl = self._pos(qubit_high, "Apply2QubitGate"), self._pos(qubit_low, "Apply2QubitGate")
        if qubit_high == qubit_low:
            raise ValueError("Apply2QubitGate: qubits coincide")
        if self.fusion:
            self._enqueue(_op(_lib.OP_2Q, ph, pl, m32))
        else:
            check(lib.iqsg_apply_2q(self._h, ph, pl, dptr(m32)))
        self._count2(qubit_high, qubit_low)

    def ApplyDiagSimp(self, qubit_1: int, qubit_2: int, m) -> None:
        """The same diagonal as ApplyDiag, not counted as a gate (src/qureg_applydiag.cpp:17-51)."""
        counter, self.gate_counter = self.gate_counter, None
        try:
            self.ApplyDiag(qubit_1, qubit_2, m)
        finally:
            self.gate_counter = counter

    def ApplyDiag(self, qubit_1: int, qubit_2: int, m) -> None:
        """src/qureg_applydiag.cpp:55-227: amp *= m[k][k], k = 2 b(qubit_1) + b(qubit_2)."""
        a = np.asarray(m, dtype=np.complex128)
        if a.shape != (4, 4):
            raise ValueError("ApplyDiag: expected a 4x4 matrix")
        d = np.ascontiguousarray(np.diag(a)).view(np.float64).copy()
        p1, p2 = self._pos(qubit_1, "ApplyDiag"), self._pos(qubit_2, "ApplyDiag")
        if qubit_1 == qubit_2:
            raise ValueError("ApplyDiag: qubits coincide")
        self._count2(qubit_1, qubit_2)
        if self.fusion:
            self._enqueue(_op(_lib.OP_DIAG2, p1, p2, d))
        else:
            check(lib.iqsg_apply_diag_2q(self._h, p1, p2, dptr(d)))

    ApplyDiagonalGate = ApplyDiag

    def ApplyMultiControlled1QubitGate(self, controls: Sequence[int], target: int, m) -> None:
        """2x2 gate on target where every control qubit is 1, in one pass."""
        m8 = _m2(m)
        check_distinct(list(controls) + [target], self._n, "ApplyMultiControlled1QubitGate")
        pc = np.asarray([self.qubit_permutation.map[c] for c in controls], dtype=np.uint32)
        if self.fusion and len(pc) <= 4:
            self._enqueue(_op(_lib.OP_CTRL, self.qubit_permutation.map[target], 0, m8, ctrl=[int(c) for c in pc]))
            return
        self._flush()
        check(lib.iqsg_apply_multi_controlled_1q(self._h, len(pc), uptr(pc), self.qubit_permutation.map[target],
                                                 dptr(m8)))

    # ---- named one-qubit gates ----------------------------------------------------------------
    def ApplyRotationX(self, qubit: int, theta: float) -> None:
        t = self._bt(theta)
        s, c = math.sin(t / 2.0), math.cos(t / 2.0)
        self.Apply1QubitGate(qubit, [[c, complex(0, -s)], [complex(0, -s), c]])

    def ApplyRotationY(self, qubit: int, theta: float) -> None:
        t = self._bt(theta)
        s, c = math.sin(t / 2.0), math.cos(t / 2.0)
        self.Apply1QubitGate(qubit, [[c, -s], [s, c]])

    def ApplyRotationZ(self, qubit: int, theta: float) -> None:
        t = self._bt(theta)
        s, c = math.sin(t / 2.0), math.cos(t / 2.0)
        self.Apply1QubitGate(qubit, [[complex(c, -s), 0], [0, complex(c, s)]])

    def ApplyPauliX(self, qubit: int) -> None:
        self.Apply1QubitGate(qubit, [[0, 1], [1, 0]])

    def ApplyPauliY(self, qubit: int) -> None:
        self.Apply1QubitGate(qubit, [[0, -1j], [1j, 0]])

    def ApplyPauliZ(self, qubit: int) -> None:
        self.Apply1QubitGate(qubit, [[1, 0], [0, -1]])

    def ApplyPauliSqrtX(self, qubit: int) -> None:
        self.Apply1QubitGate(qubit, [[0.5 + 0.5j, 0.5 - 0.5j], [0.5 - 0.5j, 0.5 + 0.5j]])

    def ApplyPauliSqrtY(self, qubit: int) -> None:
        self.Apply1QubitGate(qubit, [[0.5 + 0.5j, -0.5 - 0.5j], [0.5 + 0.5j, 0.5 + 0.5j]])

    def ApplyPauliSqrtZ(self, qubit: int) -> None:
        self.Apply1QubitGate(qubit, [[1, 0], [0, 1j]])

    def ApplyT(self, qubit: int) -> None:
        self.Apply1QubitGate(qubit, [[1, 0], [0, complex(math.cos(math.pi / 4.0), math.sin(math.pi / 4.0))]])

    def ApplyHadamard(self, qubit: int) -> None:
        f = self._bt(1.0 / math.sqrt(2.0))
        self.Apply1QubitGate(qubit, [[f, f], [f, -f]])

    def ApplyRotationXY(self, qubit: int, phi: float, theta: float) -> None:
        p, t = self._bt(phi), self._bt(theta)
        s, c = math.sin(t / 2.0), math.cos(t / 2.0)
        self.Apply1QubitGate(qubit, [[complex(c, 0), complex(-s * math.sin(p), -s * math.cos(p))],
                                     [complex(s * math.sin(p), -s * math.cos(p)), complex(c, 0)]])

    # ---- named controlled gates -----------------------------------------------------------------
    def ApplyCRotationX(self, control: int, target: int, theta: float) -> None:
        t = self._bt(theta)
        s, c = math.sin(t / 2.0), math.cos(t / 2.0)
        self.ApplyControlled1QubitGate(control, target, [[c, complex(0, -s)], [complex(0, -s), c]])

    def ApplyCRotationY(self, control: int, target: int, theta: float) -> None:
        t = self._bt(theta)
        s, c = math.sin(t / 2.0), math.cos(t / 2.0)
        self.ApplyControlled1QubitGate(control, target, [[c, -s], [s, c]])

    def ApplyCRotationZ(self, control: int, target: int, theta: float) -> None:
        t = self._bt(theta)
        s, c = math.sin(t / 2.0), math.cos(t / 2.0)
        self.ApplyControlled1QubitGate(control, target, [[complex(c, -s), 0], [0, complex(c, s)]])

    def ApplyCPauliX(self, control: int, target: int) -> None:
        self.ApplyControlled1QubitGate(control, target, [[0, 1], [1, 0]])

    def ApplyCPauliY(self, control: int, target: int) -> None:
        self.ApplyControlled1QubitGate(control, target, [[0, -1j], [1j, 0]])

    def ApplyCPauliZ(self, control: int, target: int) -> None:
        self.ApplyControlled1QubitGate(control, target, [[1, 0], [0, -1]])

    def ApplyCPauliSqrtZ(self, control: int, target: int) -> None:
        self.ApplyControlled1QubitGate(control, target, [[1, 0], [0, 1j]])

    def ApplyCHadamard(self, control: int, target: int) -> None:
        f = self._bt(1.0 / math.sqrt(2.0))
        self.ApplyControlled1QubitGate(control, target, [[f, f], [f, -f]])

    def ApplyCPhaseRotation(self, control: int, target: int, theta: float) -> None:
        """diag(1, e^{i theta}) on target when control is 1 (src/qureg_applyctrl1qubitgate.cpp:610-618)."""
        t = self._bt(theta)
        self.ApplyControlled1QubitGate(control, target, [[1, 0], [0, complex(math.cos(t), math.sin(t))]])

    # ---- swap family, Toffoli -----------------------------------------------------------------------
    def _swaplike(self, q1: int, q2: int, m, what: str) -> None:
        self._count2(q1, q2)
        p1, p2 = self._pos(q1, what), self._pos(q2, what)
        if q1 == q2:
            raise ValueError(f"{what}: qubits coincide")
        m8 = _m2(m)
        # The reference orders the two positions and asserts the block is symmetric when
        # it had to swap them (src/qureg_applyswap.cpp:140-144).
        if p1 > p2 and (m8[2] != m8[4] or m8[3] != m8[5]):
            raise ValueError(f"{what}: the 2x2 block must be symmetric (m01 == m10)")
        if self.fusion:
            self._enqueue(_op(_lib.OP_SWAPLIKE, p1, p2, m8))
        else:
            check(lib.iqsg_apply_swaplike(self._h, p1, p2, dptr(m8)))

    def ApplySwap(self, qubit1: int, qubit2: int) -> None:
        """src/qureg_applyswap.cpp:23-29."""
        self._swaplike(qubit1, qubit2, [[0, 1], [1, 0]], "ApplySwap")

    def ApplyISwap(self, qubit1: int, qubit2: int) -> None:
        self._swaplike(qubit1, qubit2, [[0, 1j], [1j, 0]], "ApplyISwap")

    def ApplySqrtISwap(self, qubit1: int, qubit2: int) -> None:
        f = self._bt(1.0 / math.sqrt(2.0))
        self._swaplike(qubit1, qubit2, [[f, 1j * f], [1j * f, f]], "ApplySqrtISwap")

    def Apply4thRootISwap(self, qubit1: int, qubit2: int) -> None:
        a = cmath.rect(0.5, math.pi / 8.0)
        b = cmath.rect(0.5, 7.0 * math.pi / 8.0)
        f0, f1 = a - b, a + b
        self._swaplike(qubit1, qubit2, [[f0, f1], [f1, f0]], "Apply4thRootISwap")

    def ApplyISwapRotation(self, qubit1: int, qubit2: int, m) -> None:
        a = np.asarray(m, dtype=np.complex128)
        if a.shape != (2, 2) or a[0, 1] != a[1, 0]:
            raise ValueError("ApplyISwapRotation: m must be 2x2 with m01 == m10")
        self._swaplike(qubit1, qubit2, a, "ApplyISwapRotation")

    def ApplyToffoli(self, control_1: int, control_2: int, target: int) -> None:
        """Flip target when both controls are 1, in one pass over the |11x> sub-block. The
        reference composes it from five controlled gates (src/qureg_applytoffoli.cpp:24-47);
        the gate counter records those five two-qubit gates as the reference does."""
        check_distinct([control_1, control_2, target], self._n, "ApplyToffoli")
        if self.gate_counter is not None:
            for a, b in ((control_1, target), (control_2, control_1), (control_1, target),
                         (control_2, control_1), (control_2, target)):
                self.gate_counter.TwoQubitIncrement(a, b)
        pc = np.asarray([self.qubit_permutation.map[control_1], self.qubit_permutation.map[control_2]], dtype=np.uint32)
        m8 = _m2([[0, 1], [1, 0]])
        if self.fusion:
            self._enqueue(_op(_lib.OP_CTRL, self.qubit_permutation.map[target], 0, m8, ctrl=[int(c) for c in pc]))
        else:
            check(lib.iqsg_apply_multi_controlled_1q(self._h, 2, uptr(pc), self.qubit_permutation.map[target],
                                                     dptr(m8)))

    # ---- permutation of the qubit order ---------------------------------------------------------------
    def PermuteQubits(self, new_map: Sequence[int], style_of_map: str = "direct") -> None:
        """src/qureg_permute.cpp:10-41 (one device reorder: no local/global split on one GPU)."""
        if len(new_map) != self._n:
            raise ValueError(f"PermuteQubits: map has {len(new_map)} entries for {self._n} qubits")
        new = Permutation(list(new_map), style_of_map)
        old = np.asarray(self.qubit_permutation.map, dtype=np.uint32)
        nm = np.asarray(new.map, dtype=np.uint32)
        check(lib.iqsg_permute(self._h, uptr(old), uptr(nm)))
        self.qubit_permutation = new

    PermuteLocalQubits = PermuteQubits

    def EmulateSwap(self, qubit1: int, qubit2: int) -> None:
        """src/qureg_permute.cpp:45-53: swap by relabelling, no data movement."""
        check_distinct([qubit1], self._n, "EmulateSwap")
        check_distinct([qubit2], self._n, "EmulateSwap")
        self.qubit_permutation.ExchangeTwoElements(qubit1, qubit2)

    # ---- measurement ---------------------------------------------------------------------------------
    def GetProbability(self, qubit: int) -> float:
        """Probability of |1> on qubit, unnormalised (src/qureg_measure.cpp:135-178)."""
        p = C.c_double()
        check(lib.iqsg_probability(self._h, self._pos(qubit, "GetProbability"), C.byref(p)))
        return p.value

    def CollapseQubit(self, qubit: int, value: bool) -> None:
        """src/qureg_measure.cpp:92-126 (no renormalisation)."""
        check(lib.iqsg_collapse(self._h, self._pos(qubit, "CollapseQubit"), 1 if value else 0))

    def IsClassicalBit(self, qubit: int, tolerance: float = 1.e-13) -> bool:
        """src/qureg_measure.cpp:19-81: probability of |1> within tolerance of 0 or 1."""
        p = self.GetProbability(qubit)
        return p < tolerance or abs(1.0 - p) < tolerance

    def GetClassicalValue(self, qubit: int, tolerance: float = 1.e-13) -> bool:
        p = self.GetProbability(qubit)
        if p < tolerance:
            return False
        if abs(1.0 - p) < tolerance:
            return True
        raise ValueError(f"GetClassicalValue: qubit {qubit} is not classical (P(1) = {p})")

    # ---- expectation values -----------------------------------------------------------------------------
    def ExpectationValue(self, qubits: Sequence[int], observables: Sequence[int], coeff: float = 1.0) -> float:
        """coeff * <psi|P|psi> for P = prod_k observables[k] on qubits[k] (1 = X, 2 = Y, 3 = Z),
        unnormalised, in one read-only pass (src/qureg_expectval.cpp:102-213). A single-factor
        string returns coeff * (1 - 2 P(1)) in the rotated basis, as the reference's
        ExpectationValueX/Y/Z do (src/qureg_expectval.cpp:18-75)."""
        qubits, observables = list(qubits), list(observables)
        if len(qubits) != len(observables):
            raise ValueError("ExpectationValue: qubits and observables differ in length")
        for o in observables:
            if o not in (1, 2, 3):
                raise ValueError(f"ExpectationValue: observable {o} not in {{1, 2, 3}}")
        check_distinct(qubits, self._n, "ExpectationValue")
        if not qubits:
            return self._bt(coeff)
        if self.gate_counter is not None:  # the reference's basis changes and their undo
            for q, o in zip(qubits, observables):
                if o in (1, 2):
                    self.gate_counter.OneQubitIncrement(q)
            for q, o in zip(qubits, observables):
                if o in (1, 2):
                    self.gate_counter.OneQubitIncrement(q)
        pos = np.asarray([self.qubit_permutation.map[q] for q in qubits], dtype=np.uint32)
        obs = np.asarray(observables, dtype=np.uint32)
        val, n2 = C.c_double(), C.c_double()
        check(lib.iqsg_expectation_pauli(self._h, len(pos), uptr(pos), uptr(obs), C.byref(val), C.byref(n2)))
        e = val.value if len(qubits) > 1 else 1.0 - n2.value + val.value
        return self._bt(coeff) * e

    def ExpectationValueX(self, qubit: int, coeff: float = 1.0) -> float:
        return self.ExpectationValue([qubit], [1], coeff)

    def ExpectationValueY(self, qubit: int, coeff: float = 1.0) -> float:
        return self.ExpectationValue([qubit], [2], coeff)

    def ExpectationValueZ(self, qubit: int, coeff: float = 1.0) -> float:
        return self.ExpectationValue([qubit], [3], coeff)

    def _ev2(self, a, b, q1, q2, coeff):
        return self.ExpectationValue([q1, q2], [a, b], coeff)

    def ExpectationValueXX(self, q1, q2, coeff=1.0): return self._ev2(1, 1, q1, q2, coeff)
    def ExpectationValueXY(self, q1, q2, coeff=1.0): return self._ev2(1, 2, q1, q2, coeff)
    def ExpectationValueXZ(self, q1, q2, coeff=1.0): return self._ev2(1, 3, q1, q2, coeff)
    def ExpectationValueYX(self, q1, q2, coeff=1.0): return self._ev2(2, 1, q1, q2, coeff)
    def ExpectationValueYY(self, q1, q2, coeff=1.0): return self._ev2(2, 2, q1, q2, coeff)
    def ExpectationValueYZ(self, q1, q2, coeff=1.0): return self._ev2(2, 3, q1, q2, coeff)
    def ExpectationValueZX(self, q1, q2, coeff=1.0): return self._ev2(3, 1, q1, q2, coeff)
    def ExpectationValueZY(self, q1, q2, coeff=1.0): return self._ev2(3, 2, q1, q2, coeff)
    def ExpectationValueZZ(self, q1, q2, coeff=1.0): return self._ev2(3, 3, q1, q2, coeff)

    # ---- norms, overlaps, amplitude-wise operations ----------------------------------------------------------
    def _same_layout(self, other: "QubitRegister", what: str) -> None:
        if not isinstance(other, QubitRegister):
            raise TypeError(f"{what}: expected a QubitRegister")
        if other.qubit_permutation.map != self.qubit_permutation.map:
            raise ValueError(f"{what}: the two registers have different qubit orders")

    def ComputeNorm(self) -> float:
        """src/qureg_utils.cpp:236-256."""
        v = C.c_double()
        check(lib.iqsg_norm2(self._h, C.byref(v)))
        return self._bt(math.sqrt(v.value))

    def Normalize(self) -> None:
        """src/qureg_utils.cpp:162-169."""
        nrm = self.ComputeNorm()
        self.AmplitudeWiseScalarMultiplication(complex(self._bt(1.0 / nrm), 0.0))

    def ComputeOverlap(self, psi: "QubitRegister") -> complex:
        """<psi|this> (src/qureg_utils.cpp:267-300)."""
        self._same_layout(psi, "ComputeOverlap")
        out = (C.c_double * 2)()
        check(lib.iqsg_overlap(self._h, psi._h, out))
        return complex(out[0], out[1])

    def MaxAbsDiff(self, x: "QubitRegister", sfactor: complex = 1.0) -> float:
        """src/qureg_utils.cpp:40-68."""
        self._same_layout(x, "MaxAbsDiff")
        s = complex(sfactor)
        v = C.c_double()
        check(lib.iqsg_max_abs_diff(self._h, x._h, s.real, s.imag, C.byref(v)))
        return v.value

    def MaxL2NormDiff(self, x: "QubitRegister") -> float:
        """src/qureg_utils.cpp:129-157 (sum of squared differences, no square root)."""
        self._same_layout(x, "MaxL2NormDiff")
        v = C.c_double()
        check(lib.iqsg_l2_diff(self._h, x._h, C.byref(v)))
        return v.value

    def AmplitudeWiseScalarMultiplication(self, factor: complex) -> None:
        f = complex(factor)
        check(lib.iqsg_scale(self._h, f.real, f.imag))

    def AmplitudeWiseSum(self, psi: "QubitRegister", factor: complex = 1.0) -> None:
        self._same_layout(psi, "AmplitudeWiseSum")
        f = complex(factor)
        check(lib.iqsg_axpy(self._h, psi._h, f.real, f.imag))

    def __eq__(self, other) -> bool:
        if not isinstance(other, QubitRegister) or other._n != self._n or other._prec != self._prec:
            return False
        return self.MaxAbsDiff(other) == 0.0

    __hash__ = None

    def __repr__(self) -> str:
        return f"<QubitRegister {self._n} qubits {self.precision} on GPU>"


def _flushing(fn):
    """Apply queued (fused) gates of every register argument before fn reads or changes
    the state outside the gate stream."""
    import functools

    @functools.wraps(fn)
    def wrapper(self, *args, **kwargs):
        if self._queue:
            self._flush()
        for a in args:
            if isinstance(a, QubitRegister) and a._queue:
                a._flush()
        return fn(self, *args, **kwargs)
    return wrapper


for _name in ("SetMath", "RawState", "synchronize", "Initialize", "InitializationWithSameAmplitudeEverywhere",
              "GetStateVector", "SetStateVector", "__getitem__", "__setitem__", "PermuteQubits", "GetProbability",
              "CollapseQubit", "IsClassicalBit", "GetClassicalValue", "ExpectationValue", "ComputeNorm", "Normalize",
              "ComputeOverlap", "MaxAbsDiff", "MaxL2NormDiff", "AmplitudeWiseScalarMultiplication",
              "AmplitudeWiseSum", "__eq__"):
    setattr(QubitRegister, _name, _flushing(getattr(QubitRegister, _name)))
QubitRegister.PermuteLocalQubits = QubitRegister.PermuteQubits


def plan_ops(num_qubits: int, ops, *, precision: str = "DP", math: str = "native", width: int = 0) -> dict:
    """The fused sweeps iqsg_apply_ops would run for a list of `_lib.Op` gates on a register of
    num_qubits positions (host only; no GPU needed): {"sweeps": [{"k", "positions", "ops",
    "one_qubit", "two_qubit", "diagonal"}, ...], "pair_storage": bool}."""
    arr = (_lib.Op * max(1, len(ops)))(*ops)
    n = C.c_uint()
    pairs = C.c_int()
    check(lib.iqsg_plan_ops(int(num_qubits), _PREC[precision], _MATH[math], int(width), C.cast(arr, C.c_void_p),
                            len(ops), None, 0, C.byref(n), C.byref(pairs)))
    info = (_lib.SweepInfo * max(1, n.value))()
    check(lib.iqsg_plan_ops(int(num_qubits), _PREC[precision], _MATH[math], int(width), C.cast(arr, C.c_void_p),
                            len(ops), info, n.value, C.byref(n), C.byref(pairs)))
    sweeps = [{"k": s.k, "positions": list(s.pos)[:s.k], "ops": s.ops, "one_qubit": s.one_qubit,
               "two_qubit": s.two_qubit, "diagonal": s.diagonal} for s in info[:n.value]]
    return {"sweeps": sweeps, "pair_storage": bool(pairs.value)}

