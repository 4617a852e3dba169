"""CPU oracle for the state-vector hot path -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU legs import this package, and only
as the checker (or the timed CPU baseline). The product (iqs_gb300 / libiqsg) never
imports, links or calls anything here.

Two backends with the same method names as iqs::QubitRegister<Type>:
  OracleRegister -- the plain-C restatement in iqs_oracle.c (built into _build/), plus a
                    Python restatement of the register's host logic (program qubit ->
                    position map, named-gate matrices, expectation-value basis changes).
                    It travels to any machine and is pinned against the golden vectors in
                    tests/golden/, which were produced by the reference itself.
  RefRegister    -- the reference library itself (its own sources compiled into
                    _ref/libiqs_ref.so with ref_capi.cpp); available only where the
                    reference sources exist, used to generate and check golden vectors.
"""
from __future__ import annotations

import cmath
import ctypes as C
import math
import os
import subprocess
from pathlib import Path
from typing import Sequence

import numpy as np

HERE = Path(__file__).resolve().parent
ORACLE_LIB = HERE / "_build" / "liboracle.so"
REF_LIB = HERE / "_ref" / "libiqs_ref.so"
REF_SRC = Path(os.environ.get("IQS_REFERENCE_DIR", "/root/reference"))

_P, _U, _D, _DP, _UP, _IP = C.c_void_p, C.c_uint, C.c_double, C.POINTER(C.c_double), C.POINTER(C.c_uint), C.POINTER(C.c_int)


def build(ref: bool | None = None) -> None:
    """Compile the C restatement; also the reference library when its sources are here."""
    subprocess.run(["make", "-s", "-C", str(HERE), "all"], check=True)
    if ref is None:
        ref = (REF_SRC / "src" / "qureg_init.cpp").exists()
    if ref:
        subprocess.run(["make", "-s", "-C", str(HERE), "ref", f"REF={REF_SRC}"], check=True)


_olib = None


def olib() -> C.CDLL:
    global _olib
    if _olib is None:
        if not ORACLE_LIB.exists():
            build(ref=False)
        L = C.CDLL(str(ORACLE_LIB))
        for S, T in (("d", C.c_double), ("f", C.c_float)):
            TP = C.POINTER(T)
            sig = {
                "apply1q": ([TP, _U, _U, _DP], None), "ctrl1q": ([TP, _U, _U, _U, _DP], None),
                "apply2q": ([TP, _U, _U, _U, _DP], None), "swaplike": ([TP, _U, _U, _U, _DP], None),
                "diag2": ([TP, _U, _U, _U, _DP], None), "permute": ([TP, _U, _UP, _UP], None),
                "probability": ([TP, _U, _U], _D), "collapse": ([TP, _U, _U, C.c_int], None),
                "parity_sum": ([TP, _U, C.c_uint64], _D), "norm": ([TP, _U], _D),
                "overlap": ([TP, TP, _U, _DP], None), "max_abs_diff": ([TP, TP, _U, _D, _D], _D),
                "max_l2_diff": ([TP, TP, _U], _D), "scale": ([TP, _U, _D, _D], None),
                "axpy": ([TP, TP, _U, _D, _D], None), "fill": ([TP, _U, _D, _D], None),
                "qaoa_layer": ([TP, TP, _U, _D], None), "qaoa_expectation": ([TP, TP, _U], _D),
                "qaoa_expectation_sq": ([TP, TP, _U], _D), "qaoa_maxcut_cost": ([TP, _U, _IP, _UP], C.c_int),
                "qaoa_weighted_cost": ([TP, _U, _DP, _UP], _D),
            }
            for name, (args, res) in sig.items():
                fn = getattr(L, f"or_{name}_{S}")
                fn.argtypes = args
                fn.restype = res
        L.or_set_threads.argtypes = [C.c_int]
        L.or_get_threads.restype = C.c_int
        _olib = L
    return _olib


def set_threads(n: int) -> None:
    olib().or_set_threads(int(n))


def get_threads() -> int:
    return olib().or_get_threads()


# ---------------------------------------------------------------------------------------
# Named-gate matrices and host logic, restated from the reference sources cited.
# ---------------------------------------------------------------------------------------
def _h(bt):
    f = bt(1.0 / math.sqrt(2.0))
    return [[f, f], [f, -f]]


def _rx(t):
    s, c = math.sin(t / 2.0), math.cos(t / 2.0)
    return [[c, complex(0, -s)], [complex(0, -s), c]]


def _ry(t):
    s, c = math.sin(t / 2.0), math.cos(t / 2.0)
    return [[c, -s], [s, c]]


def _rz(t):
    s, c = math.sin(t / 2.0), math.cos(t / 2.0)
    return [[complex(c, -s), 0], [0, complex(c, s)]]


# src/qureg_apply1qubitgate.cpp:277-501 and src/qureg_applyctrl1qubitgate.cpp:458-618
FIXED_1Q = {
    "ApplyPauliX": [[0, 1], [1, 0]],
    "ApplyPauliY": [[0, -1j], [1j, 0]],
    "ApplyPauliZ": [[1, 0], [0, -1]],
    "ApplyPauliSqrtX": [[0.5 + 0.5j, 0.5 - 0.5j], [0.5 - 0.5j, 0.5 + 0.5j]],
    "ApplyPauliSqrtY": [[0.5 + 0.5j, -0.5 - 0.5j], [0.5 + 0.5j, 0.5 + 0.5j]],
    "ApplyPauliSqrtZ": [[1, 0], [0, 1j]],
    "ApplyT": [[1, 0], [0, complex(math.cos(math.pi / 4.0), math.sin(math.pi / 4.0))]],
}
FIXED_C1Q = {
    "ApplyCPauliX": [[0, 1], [1, 0]],
    "ApplyCPauliY": [[0, -1j], [1j, 0]],
    "ApplyCPauliZ": [[1, 0], [0, -1]],
    "ApplyCPauliSqrtZ": [[1, 0], [0, 1j]],
}


class _Perm:
    """include/permutation.hpp: map (qubit -> position) and imap."""

    def __init__(self, n):
        self.map = list(range(n))

    def set(self, m, style):
        n = len(m)
        assert sorted(m) == list(range(n)), "not a permutation"
        if style == "direct":
            self.map = list(m)
        else:
            mp = [0] * n
            for p, q in enumerate(m):
                mp[q] = p
            self.map = mp

    @property
    def imap(self):
        im = [0] * len(self.map)
        for q, p in enumerate(self.map):
            im[p] = q
        return im

    def program2data_(self, v):
        out = 0
        for p, q in enumerate(self.imap):
            out |= ((v >> q) & 1) << p
        return out


class _Named:
    """Named gates in terms of Apply1QubitGate / ApplyControlled1QubitGate / swap helper,
    with the matrices the reference builds (float-rounded angles for ComplexSP)."""

    def _bt(self, x):
        return float(np.float32(x)) if self.sp else float(x)

    def ApplyRotationX(self, q, t): self.Apply1QubitGate(q, _rx(self._bt(t)))
    def ApplyRotationY(self, q, t): self.Apply1QubitGate(q, _ry(self._bt(t)))
    def ApplyRotationZ(self, q, t): self.Apply1QubitGate(q, _rz(self._bt(t)))
    def ApplyHadamard(self, q): self.Apply1QubitGate(q, _h(self._bt))

    def ApplyRotationXY(self, q, phi, theta):
        p, t = self._bt(phi), self._bt(theta)
        s, c = math.sin(t / 2.0), math.cos(t / 2.0)
        self.Apply1QubitGate(q, [[c, complex(-s * math.sin(p), -s * math.cos(p))],
                                 [complex(s * math.sin(p), -s * math.cos(p)), c]])

    def ApplyCRotationX(self, c, t, th): self.ApplyControlled1QubitGate(c, t, _rx(self._bt(th)))
    def ApplyCRotationY(self, c, t, th): self.ApplyControlled1QubitGate(c, t, _ry(self._bt(th)))
    def ApplyCRotationZ(self, c, t, th): self.ApplyControlled1QubitGate(c, t, _rz(self._bt(th)))
    def ApplyCHadamard(self, c, t): self.ApplyControlled1QubitGate(c, t, _h(self._bt))

    def ApplyCPhaseRotation(self, c, t, th):
        th = self._bt(th)
        self.ApplyControlled1QubitGate(c, t, [[1, 0], [0, complex(math.cos(th), math.sin(th))]])

    def __getattr__(self, name):
        if name in FIXED_1Q:
            return lambda q: self.Apply1QubitGate(q, FIXED_1Q[name])
        if name in FIXED_C1Q:
            return lambda c, t: self.ApplyControlled1QubitGate(c, t, FIXED_C1Q[name])
        raise AttributeError(name)

    def ApplySwap(self, a, b): self._swap(a, b, [[0, 1], [1, 0]])
    def ApplyISwap(self, a, b): self._swap(a, b, [[0, 1j], [1j, 0]])

    def ApplySqrtISwap(self, a, b):
        f = self._bt(1.0 / math.sqrt(2.0))
        self._swap(a, b, [[f, 1j * f], [1j * f, f]])

    def Apply4thRootISwap(self, a, b):
        x, y = cmath.rect(0.5, math.pi / 8.0), cmath.rect(0.5, 7.0 * math.pi / 8.0)
        self._swap(a, b, [[x - y, x + y], [x + y, x - y]])

    def ApplyISwapRotation(self, a, b, m): self._swap(a, b, m)

    def ApplyToffoli(self, c1, c2, t):
        """src/qureg_applytoffoli.cpp:24-47: five controlled gates."""
        V = [[0.5 - 0.5j, 0.5 + 0.5j], [0.5 + 0.5j, 0.5 - 0.5j]]
        Vd = [[0.5 + 0.5j, 0.5 - 0.5j], [0.5 - 0.5j, 0.5 + 0.5j]]
        self.ApplyControlled1QubitGate(c1, t, V)
        self.ApplyCPauliX(c2, c1)
        self.ApplyControlled1QubitGate(c1, t, Vd)
        self.ApplyCPauliX(c2, c1)
        self.ApplyControlled1QubitGate(c2, t, V)

    def ExpectationValueX(self, q, coeff=1.0): return self.ExpectationValue([q], [1], coeff)
    def ExpectationValueY(self, q, coeff=1.0): return self.ExpectationValue([q], [2], coeff)
    def ExpectationValueZ(self, q, coeff=1.0): return self.ExpectationValue([q], [3], coeff)
    def ExpectationValueZZ(self, a, b, coeff=1.0): return self.ExpectationValue([a, b], [3, 3], coeff)
    def ExpectationValueXX(self, a, b, coeff=1.0): return self.ExpectationValue([a, b], [1, 1], coeff)
    def ExpectationValueYY(self, a, b, coeff=1.0): return self.ExpectationValue([a, b], [2, 2], coeff)


def _m(m, k):
    a = np.ascontiguousarray(np.asarray(m, dtype=np.complex128).reshape(k, k))
    return a.reshape(-1).view(np.float64).copy()


class OracleRegister(_Named):
    """QubitRegister restated over the C oracle (iqs_oracle.c); state in host memory."""

    def __init__(self, n, style="base", base_index=0, precision="DP"):
        self.n = int(n)
        self.sp = precision == "SP"
        self.s = np.zeros(1 << self.n, dtype=np.complex64 if self.sp else np.complex128)
        self.perm = _Perm(self.n)
        self.L = olib()
        self.S = "f" if self.sp else "d"
        self.Initialize(style, base_index)

    def _f(self, name):
        return getattr(self.L, f"or_{name}_{self.S}")

    def _p(self, a=None):
        a = self.s if a is None else a
        return a.ctypes.data_as(C.POINTER(C.c_float if self.sp else C.c_double))

    def _pos(self, q):
        return self.perm.map[q]

    def Initialize(self, style="", base_index=0):
        self.s[:] = 0
        if style == "base":
            self.s[self.perm.program2data_(base_index)] = 1.0
        elif style == "++++":
            self.s[:] = self._bt(1.0 / math.sqrt(1 << self.n))

    def NumQubits(self):
        return self.n

    def GetStateVector(self):
        return self.s.copy()

    def SetStateVector(self, a):
        self.s[:] = np.asarray(a, dtype=self.s.dtype)

    def Apply1QubitGate(self, q, m):
        self._f("apply1q")(self._p(), self.n, self._pos(q), _m(m, 2).ctypes.data_as(_DP))

    def ApplyControlled1QubitGate(self, c, t, m):
        assert c != t
        self._f("ctrl1q")(self._p(), self.n, self._pos(c), self._pos(t), _m(m, 2).ctypes.data_as(_DP))

    def Apply2QubitGate(self, qh, ql, m):
        self._f("apply2q")(self._p(), self.n, self._pos(qh), self._pos(ql), _m(m, 4).ctypes.data_as(_DP))

    def ApplyDiag(self, q1, q2, m):
        d = np.ascontiguousarray(np.diag(np.asarray(m, dtype=np.complex128))).view(np.float64).copy()
        self._f("diag2")(self._p(), self.n, self._pos(q1), self._pos(q2), d.ctypes.data_as(_DP))

    def _swap(self, a, b, m):
        self._f("swaplike")(self._p(), self.n, self._pos(a), self._pos(b), _m(m, 2).ctypes.data_as(_DP))

    def PermuteQubits(self, new_map, style="direct"):
        old = np.asarray(self.perm.map, dtype=np.uint32)
        p = _Perm(self.n)
        p.set(list(new_map), style)
        new = np.asarray(p.map, dtype=np.uint32)
        self._f("permute")(self._p(), self.n, old.ctypes.data_as(_UP), new.ctypes.data_as(_UP))
        self.perm = p

    def EmulateSwap(self, a, b):
        self.perm.map[a], self.perm.map[b] = self.perm.map[b], self.perm.map[a]

    def GetProbability(self, q):
        return self._bt(self._f("probability")(self._p(), self.n, self._pos(q)))

    def CollapseQubit(self, q, v):
        self._f("collapse")(self._p(), self.n, self._pos(q), 1 if v else 0)

    def ExpectationValue(self, qubits, obs, coeff=1.0):
        """src/qureg_expectval.cpp:102-213: basis change, parity reduction, undo."""
        qubits, obs = list(qubits), list(obs)
        if not qubits:
            return self._bt(coeff)
        f = self._bt(1.0 / math.sqrt(2.0))
        G = [[f, complex(0, -f)], [f, complex(0, f)]]
        Gi = [[f, f], [complex(0, f), complex(0, -f)]]
        if len(qubits) == 1:
            q, o = qubits[0], obs[0]
            if o == 1:
                self.ApplyHadamard(q)
            elif o == 2:
                self.Apply1QubitGate(q, G)
            e = self._bt(1.0 - 2.0 * self.GetProbability(q))
            if o == 1:
                self.ApplyHadamard(q)
            elif o == 2:
                self.Apply1QubitGate(q, Gi)
            return self._bt(self._bt(coeff) * e)
        for q, o in zip(qubits, obs):
            if o == 1:
                self.ApplyHadamard(q)
            elif o == 2:
                self.Apply1QubitGate(q, G)
        mask = 0
        for q in qubits:
            mask += 1 << self._pos(q)
        e = self._f("parity_sum")(self._p(), self.n, mask)
        for q, o in zip(qubits, obs):
            if o == 1:
                self.ApplyHadamard(q)
            elif o == 2:
                self.Apply1QubitGate(q, Gi)
        return self._bt(self._bt(coeff) * self._bt(e))

    def ComputeNorm(self):
        return self._f("norm")(self._p(), self.n)

    def Normalize(self):
        self.AmplitudeWiseScalarMultiplication(self._bt(1.0 / self.ComputeNorm()))

    def ComputeOverlap(self, psi):
        out = (C.c_double * 2)()
        self._f("overlap")(self._p(), self._p(psi.s), self.n, out)
        return complex(out[0], out[1])

    def MaxAbsDiff(self, x, sfactor=1.0):
        s = complex(sfactor)
        return self._f("max_abs_diff")(self._p(), self._p(x.s), self.n, s.real, s.imag)

    def MaxL2NormDiff(self, x):
        return self._f("max_l2_diff")(self._p(), self._p(x.s), self.n)

    def AmplitudeWiseScalarMultiplication(self, f):
        f = complex(f)
        self._f("scale")(self._p(), self.n, f.real, f.imag)

    def AmplitudeWiseSum(self, psi, f=1.0):
        f = complex(f)
        self._f("axpy")(self._p(), self._p(psi.s), self.n, f.real, f.imag)

    def InitializationWithSameAmplitudeEverywhere(self, a):
        a = complex(a)
        self._f("fill")(self._p(), self.n, a.real, a.imag)

    def GetGlobalAmplitude(self, idx):
        return complex(self.s[self.perm.program2data_(idx)])

    def SetGlobalAmplitude(self, idx, v):
        self.s[self.perm.program2data_(idx)] = v

    def __getitem__(self, i):
        return complex(self.s[i])

    def __setitem__(self, i, v):
        self.s[i] = v


def oracle_maxcut_cost(diag: OracleRegister, adjacency) -> int:
    adj = np.ascontiguousarray(np.asarray(adjacency, dtype=np.int32).reshape(-1))
    mp = np.asarray(diag.perm.map, dtype=np.uint32)
    return diag._f("qaoa_maxcut_cost")(diag._p(), diag.n, adj.ctypes.data_as(_IP), mp.ctypes.data_as(_UP))


def oracle_qaoa_layer(psi: OracleRegister, diag: OracleRegister, gamma: float) -> None:
    psi._f("qaoa_layer")(psi._p(), psi._p(diag.s), psi.n, psi._bt(gamma))


def oracle_qaoa_expectation(psi: OracleRegister, diag: OracleRegister, power: int = 1) -> float:
    name = "qaoa_expectation" if power == 1 else "qaoa_expectation_sq"
    return psi._f(name)(psi._p(), psi._p(diag.s), psi.n)


# ---------------------------------------------------------------------------------------
# The reference itself (only where its sources were compiled into _ref/).
# ---------------------------------------------------------------------------------------
_rlib = None


def oracle_weighted_maxcut_cost(diag: OracleRegister, adjacency) -> float:
    """InitializeVectorAsWeightedMaxCutCostFunction through the C restatement."""
    adj = np.ascontiguousarray(np.asarray(adjacency, dtype=np.float64).reshape(-1))
    mp = np.asarray(diag.perm.map, dtype=np.uint32)
    return float(diag._f("qaoa_weighted_cost")(diag._p(), diag.n, adj.ctypes.data_as(_DP), mp.ctypes.data_as(_UP)))


def oracle_cost_histogram(psi: OracleRegister, diag: OracleRegister, mode: int, max_value: float,
                          bin_width: float = 1.0) -> np.ndarray:
    """The three histogram functions of src/qaoa_features.cpp:335-538 restated with numpy:
    mode 0 bins (int)cost over 0..max_value; mode 1 floor(cost + 1e-7) over
    0..floor(max_value); mode 2 floor(cost / bin_width + 1e-7) over 0..ceil(max_value /
    bin_width). Sums of |psi|^2 in FP64. Raises where the reference asserts."""
    cost = diag.GetStateVector().real.astype(np.float64)
    p = np.abs(psi.GetStateVector().astype(np.complex128)) ** 2
    if mode == 0:
        b = np.trunc(cost).astype(np.int64)
        nb = int(max_value) + 1
        ok = (b >= 0) & (b <= max_value)
    else:
        ok = (cost >= -1e-7) & (cost <= max_value + 1e-7)
        if mode == 1:
            b = np.floor(cost + 1e-7).astype(np.int64)
            nb = int(np.floor(max_value)) + 1
        else:
            b = np.floor(cost / bin_width + 1e-7).astype(np.int64)
            nb = int(np.ceil(max_value / bin_width)) + 1
    if not np.all(ok) or np.any(b >= nb):
        raise ValueError("cost value outside the histogram range")
    return np.bincount(b, weights=p, minlength=nb)[:nb]


def oracle_uniform_random(seed: int, skip: int, count: int, a: float, b: float, precision: str = "DP") -> np.ndarray:
    """The numbers of the reference's RandomNumberGenerator stream (src/rng_utils.cpp:84-160):
    std::mt19937 seeded with seed (the 32-bit init_genrand seeding, as numpy's legacy seeding),
    std::uniform_real_distribution over it as the C++ standard library computes it -- for
    double two 32-bit draws, u = (g1 + g2 2^32) / 2^64 in double; for float one draw,
    u = float(g1) / 2^32 -- then a + (b - a) u in the same type; the first `skip` values are
    dropped."""
    bg = np.random.MT19937()
    bg._legacy_seeding(int(seed) & 0xFFFFFFFF)
    if precision == "DP":
        raw = bg.random_raw(2 * (skip + count)).astype(np.float64).reshape(-1, 2)
        u = (raw[:, 0] + raw[:, 1] * 4294967296.0) / 18446744073709551616.0
        u = np.where(u >= 1.0, np.nextafter(1.0, 0.0), u)[skip:]
        return a + (b - a) * u
    raw = bg.random_raw(skip + count).astype(np.float32)
    u = raw / np.float32(4294967296.0)
    u = np.where(u >= np.float32(1.0), np.nextafter(np.float32(1.0), np.float32(0.0)), u)[skip:]
    return np.float32(a) + (np.float32(b) - np.float32(a)) * u


def oracle_google_stats(reg: OracleRegister) -> list:
    """GoogleStats (src/qureg_utils.cpp:349-450) restated with numpy: entropy, average
    self-information and the scaled moments m2..m10 of p = |amp|^2."""
    a = reg.GetStateVector().astype(np.complex128)
    p = a.real * a.real + a.imag * a.imag
    nz = p[p != 0]
    two2n = float(p.size)
    out = [float(-np.sum(nz * np.log(nz)) / math.log(2.0)), float(-np.sum(np.log(nz)) / math.log(2.0) / two2n)]
    fact = 1.0
    for k in range(2, 11):
        fact *= k
        out.append(float(np.sum(p ** k) * (two2n ** (k - 1) / fact)))
    return out


def ref_available() -> bool:
    return REF_LIB.exists()


def rlib() -> C.CDLL:
    global _rlib
    if _rlib is None:
        L = C.CDLL(str(REF_LIB))
        sigs = {
            "ref_create": ([_U, C.c_int], _P), "ref_destroy": ([_P], None),
            "ref_set_state": ([_P, _DP], None), "ref_get_state": ([_P, _DP], None),
            "ref_initialize": ([_P, C.c_char_p, C.c_size_t], None),
            "ref_apply1q": ([_P, _U, _DP], None), "ref_ctrl1q": ([_P, _U, _U, _DP], None),
            "ref_2q": ([_P, _U, _U, _DP], None), "ref_diag": ([_P, _U, _U, _DP], None),
            "ref_iswaprot": ([_P, _U, _U, _DP], None),
            "ref_named1": ([_P, C.c_char_p, _U, _D, _D], None), "ref_named2": ([_P, C.c_char_p, _U, _U, _D], None),
            "ref_toffoli": ([_P, _U, _U, _U], None), "ref_permute": ([_P, _UP, _U, C.c_int], None),
            "ref_get_map": ([_P, _UP], None), "ref_emulate_swap": ([_P, _U, _U], None),
            "ref_get_global_amplitude": ([_P, C.c_size_t, _DP], None),
            "ref_set_global_amplitude": ([_P, C.c_size_t, _D, _D], None),
            "ref_probability": ([_P, _U], _D), "ref_collapse": ([_P, _U, C.c_int], None),
            "ref_expectation": ([_P, _U, _UP, _UP, _D], _D), "ref_norm": ([_P], _D), "ref_normalize": ([_P], None),
            "ref_overlap": ([_P, _P, _DP], None), "ref_max_abs_diff": ([_P, _P, _D, _D], _D),
            "ref_max_l2_diff": ([_P, _P], _D), "ref_scale": ([_P, _D, _D], None),
            "ref_axpy": ([_P, _P, _D, _D], None), "ref_fill": ([_P, _D, _D], None),
            "ref_fusion_on": ([_P, _U], None), "ref_fusion_off": ([_P], None),
            "ref_qaoa_maxcut_cost": ([_P, _IP, _U], C.c_int), "ref_qaoa_layer": ([_P, _P, _D], None),
            "ref_qaoa_expectation": ([_P, _P], _D), "ref_qaoa_expectation_sq": ([_P, _P], _D),
            "ref_qaoa_weighted_cost": ([_P, _DP, _U], _D),
            "ref_entropy": ([_P], _D), "ref_google_stats": ([_P, _DP, C.c_int], C.c_int),
            "ref_init_rand": ([_P, C.c_ulong, C.c_int, C.c_int], None),
            "ref_print": ([_P, C.c_char_p], None), "ref_export": ([_P, C.c_char_p], None),
            "ref_qaoa_histogram": ([_P, _P, C.c_int, _D, _D, _DP, C.c_int], C.c_int),
            "ref_rng_sequence": ([C.c_int, C.c_ulong, _IP, C.c_int, _DP, C.c_int, C.POINTER(C.c_ulong)], C.c_int),
            "ref_noise_run": ([_P, C.c_ulong, _D, _D, _UP, _DP, C.c_int, C.POINTER(C.c_ulong)], None),
            "ref_noisy_qureg_run": ([C.c_int, _U, _U, _D, _D, _D, _D, _IP, _DP, _DP, C.c_int, _DP, _UP], None),
            "ref_chi_normalize": ([C.c_int, _U, _DP, _DP, _DP, _DP, _DP], None),
            "ref_channel_run": ([_P, C.c_ulong, _U, _DP, _DP, _UP, C.c_int], _D),
            "ref_ideal_hadamard_channel": ([_P, C.c_ulong, _U, C.c_int], None),
        }
        for name, (args, res) in sigs.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _rlib = L
    return _rlib


class RefRegister:
    """The reference's QubitRegister<ComplexDP|ComplexSP>, called through ref_capi.cpp."""

    def __init__(self, n, style="base", base_index=0, precision="DP"):
        self.n = int(n)
        self.sp = precision == "SP"
        self.L = rlib()
        self.h = self.L.ref_create(self.n, 1 if self.sp else 0)
        self.Initialize(style, base_index)

    def __del__(self):
        if getattr(self, "h", None):
            self.L.ref_destroy(self.h)
            self.h = None

    def Initialize(self, style="", base_index=0):
        self.L.ref_initialize(self.h, style.encode(), base_index)

    def NumQubits(self):
        return self.n

    def GetStateVector(self):
        out = np.empty(2 << self.n, dtype=np.float64)
        self.L.ref_get_state(self.h, out.ctypes.data_as(_DP))
        v = out.view(np.complex128)
        return v.astype(np.complex64) if self.sp else v

    def SetStateVector(self, a):
        a = np.ascontiguousarray(np.asarray(a, dtype=np.complex128)).view(np.float64)
        self.L.ref_set_state(self.h, a.ctypes.data_as(_DP))

    @property
    def map(self):
        m = np.empty(self.n, dtype=np.uint32)
        self.L.ref_get_map(self.h, m.ctypes.data_as(_UP))
        return [int(x) for x in m]

    def Apply1QubitGate(self, q, m): self.L.ref_apply1q(self.h, q, _m(m, 2).ctypes.data_as(_DP))
    def ApplyControlled1QubitGate(self, c, t, m): self.L.ref_ctrl1q(self.h, c, t, _m(m, 2).ctypes.data_as(_DP))
    def Apply2QubitGate(self, qh, ql, m): self.L.ref_2q(self.h, qh, ql, _m(m, 4).ctypes.data_as(_DP))
    def ApplyDiag(self, q1, q2, m): self.L.ref_diag(self.h, q1, q2, _m(m, 4).ctypes.data_as(_DP))
    def ApplyISwapRotation(self, a, b, m): self.L.ref_iswaprot(self.h, a, b, _m(m, 2).ctypes.data_as(_DP))
    def ApplyToffoli(self, a, b, c): self.L.ref_toffoli(self.h, a, b, c)

    def __getattr__(self, name):
        one = {"ApplyRotationX", "ApplyRotationY", "ApplyRotationZ", "ApplyPauliX", "ApplyPauliY", "ApplyPauliZ",
               "ApplyPauliSqrtX", "ApplyPauliSqrtY", "ApplyPauliSqrtZ", "ApplyT", "ApplyHadamard", "ApplyRotationXY"}
        two = {"ApplyCRotationX", "ApplyCRotationY", "ApplyCRotationZ", "ApplyCPauliX", "ApplyCPauliY", "ApplyCPauliZ",
               "ApplyCPauliSqrtZ", "ApplyCHadamard", "ApplyCPhaseRotation", "ApplySwap", "ApplyISwap",
               "ApplySqrtISwap", "Apply4thRootISwap"}
        if name in one:
            return lambda q, a=0.0, b=0.0: self.L.ref_named1(self.h, name.encode(), q, a, b)
        if name in two:
            return lambda c, t, a=0.0: self.L.ref_named2(self.h, name.encode(), c, t, a)
        raise AttributeError(name)

    def PermuteQubits(self, m, style="direct"):
        a = np.asarray(m, dtype=np.uint32)
        self.L.ref_permute(self.h, a.ctypes.data_as(_UP), self.n, 1 if style == "inverse" else 0)

    def EmulateSwap(self, a, b): self.L.ref_emulate_swap(self.h, a, b)
    def GetProbability(self, q): return self.L.ref_probability(self.h, q)
    def CollapseQubit(self, q, v): self.L.ref_collapse(self.h, q, 1 if v else 0)

    def ExpectationValue(self, qubits, obs, coeff=1.0):
        q = np.asarray(qubits, dtype=np.uint32)
        o = np.asarray(obs, dtype=np.uint32)
        return self.L.ref_expectation(self.h, len(q), q.ctypes.data_as(_UP), o.ctypes.data_as(_UP), coeff)

    def ComputeNorm(self): return self.L.ref_norm(self.h)
    def Normalize(self): self.L.ref_normalize(self.h)

    def ComputeOverlap(self, psi):
        out = (C.c_double * 2)()
        self.L.ref_overlap(self.h, psi.h, out)
        return complex(out[0], out[1])

    def MaxAbsDiff(self, x, s=1.0):
        s = complex(s)
        return self.L.ref_max_abs_diff(self.h, x.h, s.real, s.imag)

    def MaxL2NormDiff(self, x): return self.L.ref_max_l2_diff(self.h, x.h)

    def AmplitudeWiseScalarMultiplication(self, f):
        f = complex(f)
        self.L.ref_scale(self.h, f.real, f.imag)

    def AmplitudeWiseSum(self, psi, f=1.0):
        f = complex(f)
        self.L.ref_axpy(self.h, psi.h, f.real, f.imag)

    def InitializationWithSameAmplitudeEverywhere(self, a):
        a = complex(a)
        self.L.ref_fill(self.h, a.real, a.imag)

    def GetGlobalAmplitude(self, idx):
        out = (C.c_double * 2)()
        self.L.ref_get_global_amplitude(self.h, idx, out)
        return complex(out[0], out[1])

    def SetGlobalAmplitude(self, idx, v):
        v = complex(v)
        self.L.ref_set_global_amplitude(self.h, idx, v.real, v.imag)

    def TurnOnFusion(self, log2llc=20): self.L.ref_fusion_on(self.h, log2llc)
    def TurnOffFusion(self): self.L.ref_fusion_off(self.h)
    def ExpectationValueZZ(self, a, b, coeff=1.0): return self.ExpectationValue([a, b], [3, 3], coeff)
