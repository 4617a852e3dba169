"""Chi matrices of quantum channels (include/chi_matrix.hpp, src/chi_matrix.cpp of intel/intel-qs):

    rho' = sum_ij chi_ij sigma_i rho sigma_j^dagger,  Pauli order {I, X, Y, Z}
    (I.I, I.X, ..., Z.Z for two qubits),

with the eigensystem chi = sum_k E_k |E_k><E_k| used by QubitRegister.ApplyChannel to pick one
Pauli-basis gate per draw with probability |E_k| / sum |E|.

SolveEigenSystem runs libiqsg's Hermitian Jacobi solver (the reference calls Eigen's
ComplexEigenSolver): eigenvalues in increasing |E_k|, each eigenvector with its largest
component real and positive. SetEigenSystem takes an eigensystem from the caller and applies the
reference's normalisation, as EigensystemOfIdealHadamardChannel does with its hand-set one.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional

import numpy as np

from . import _lib
from ._lib import check, lib

_PREC = {"DP": _lib.COMPLEX_DP, "SP": _lib.COMPLEX_SP}


def _fmt(x: float) -> str:
    return "%g" % x


def _cfmt(z: complex) -> str:
    """std::ostream << std::complex<T> with the default precision: "(re,im)"."""
    return f"({_fmt(z.real)},{_fmt(z.imag)})"


class ChiMatrix:
    def __init__(self, M: int, data=None, *, precision: str = "DP"):
        if int(M) <= 0:
            raise ValueError("A zero-dimensional matrix is not allowed.")
        if precision not in _PREC:
            raise ValueError(f"precision must be 'DP' or 'SP', not {precision!r}")
        self.M = int(M)
        self.precision = precision
        self._p = _PREC[precision]
        self._dtype = np.complex128 if precision == "DP" else np.complex64
        self.data = np.zeros((self.M, self.M), dtype=self._dtype)
        if data is not None:
            self.data[...] = np.asarray(data)
        self._evals: Optional[np.ndarray] = None
        self._evecs: Optional[np.ndarray] = None
        self._probs: Optional[np.ndarray] = None
        self._cum: Optional[np.ndarray] = None

    # ---- TinyMatrix surface ----------------------------------------------------------
    def numRows(self) -> int:
        return self.M

    def numCols(self) -> int:
        return self.M

    def size(self) -> int:
        return self.M * self.M

    def __getitem__(self, ij):
        i, j = ij
        if not (0 <= i < self.M and 0 <= j < self.M):
            raise IndexError(ij)
        return complex(self.data[i, j])

    def __setitem__(self, ij, value) -> None:
        i, j = ij
        if not (0 <= i < self.M and 0 <= j < self.M):
            raise IndexError(ij)
        self.data[i, j] = value

    def __call__(self, i: int, j: int) -> complex:
        return self[i, j]

    def __eq__(self, other) -> bool:
        return isinstance(other, ChiMatrix) and other.M == self.M and np.array_equal(other.data, self.data)

    # ---- eigensystem -------------------------------------------------------------------
    def _normalize(self, evals: np.ndarray, evecs: np.ndarray) -> None:
        M = self.M
        ev = np.ascontiguousarray(evals, dtype=np.complex128).view(np.float64)
        vecs = np.ascontiguousarray(evecs, dtype=np.complex128).reshape(M, M).copy()
        vf = vecs.view(np.float64).reshape(-1)
        probs, cum = np.zeros(M), np.zeros(M)
        check(lib.iqsg_chi_normalize(self._p, M, ev.ctypes.data_as(_lib._DP), vf.ctypes.data_as(_lib._DP),
                                     probs.ctypes.data_as(_lib._DP), cum.ctypes.data_as(_lib._DP)))
        self._evals = np.asarray(evals, dtype=np.complex128).astype(self._dtype)
        self._evecs = vecs.astype(self._dtype)
        self._probs, self._cum = probs, cum

    def SolveEigenSystem(self) -> None:
        """Eigenvalues and standardised eigenvectors (chi = sum_k E_k |E_k><E_k|), then the
        reference's normalisation (src/chi_matrix.cpp:66-127, 166-200)."""
        M = self.M
        chi = np.ascontiguousarray(self.data, dtype=np.complex128).view(np.float64).reshape(-1)
        ev = np.zeros(2 * M)
        vecs = np.zeros(2 * M * M)
        probs, cum = np.zeros(M), np.zeros(M)
        check(lib.iqsg_chi_eigensystem(self._p, M, chi.ctypes.data_as(_lib._DP), ev.ctypes.data_as(_lib._DP),
                                       vecs.ctypes.data_as(_lib._DP), probs.ctypes.data_as(_lib._DP),
                                       cum.ctypes.data_as(_lib._DP)))
        self._evals = ev.view(np.complex128).astype(self._dtype)
        self._evecs = vecs.view(np.complex128).reshape(M, M).astype(self._dtype)
        self._probs, self._cum = probs, cum

    def SetEigenSystem(self, evals, evecs) -> None:
        """Use a caller's eigensystem (row k of evecs = eigenvector k), then normalise."""
        evals = np.asarray(evals, dtype=np.complex128).reshape(-1)
        evecs = np.asarray(evecs, dtype=np.complex128)
        if evals.shape != (self.M,) or evecs.shape != (self.M, self.M):
            raise ValueError(f"eigensystem of a {self.M}x{self.M} chi matrix expected")
        self._normalize(evals.astype(self._dtype), evecs.astype(self._dtype))

    def EigensystemOfIdealHadamardChannel(self) -> None:
        """The hand-set eigensystem of the ideal Hadamard channel (src/chi_matrix.cpp:206-237): chi
        must be 0.5 on the X/Z block {1, 3} x {1, 3} and zero elsewhere; eigenvalue 1 for
        (X + Z)/sqrt(2), 0 for (X - Z)/sqrt(2), I and Y."""
        if self.M != 4:
            raise ValueError("EigensystemOfIdealHadamardChannel: 4x4 chi matrix expected")
        for i in range(4):
            for j in range(4):
                want = 0.5 if (i in (1, 3) and j in (1, 3)) else 0.0
                if self.data[i, j] != want:
                    raise ValueError("EigensystemOfIdealHadamardChannel: chi is not the ideal Hadamard channel")
        e = 1.0 / np.sqrt(2.0)
        vecs = np.array([[0, e, 0, e], [0, e, 0, -e], [1, 0, 0, 0], [0, 0, 1, 0]], dtype=np.complex128)
        self._normalize(np.array([1, 0, 0, 0], dtype=np.complex128), vecs)

    def _need(self) -> None:
        if self._evals is None:
            raise ValueError("chi matrix: no eigensystem (call SolveEigenSystem first)")

    def GetEigenValue(self, k: int) -> complex:
        self._need()
        return complex(self._evals[k])

    def GetEigenValues(self) -> list:
        self._need()
        return [complex(x) for x in self._evals]

    def GetEigenProbability(self, k: int) -> float:
        self._need()
        return float(self._probs[k])

    def GetEigenProbabilities(self) -> list:
        self._need()
        return [float(x) for x in self._probs]

    def GetEigenCumulativeProbability(self, k: int) -> float:
        self._need()
        return float(self._cum[k])

    def GetEigenCumulativeProbabilities(self) -> list:
        self._need()
        return [float(x) for x in self._cum]

    def GetEigenVector(self, k: int) -> list:
        self._need()
        return [complex(x) for x in self._evecs[k]]

    def GetEigenVectors(self) -> list:
        self._need()
        return [[complex(x) for x in row] for row in self._evecs]

    def _arrays(self):
        """(evals, cumprobs, evecs) as flat float64 arrays for iqsg_channel_gate."""
        self._need()
        ev = np.ascontiguousarray(self._evals, dtype=np.complex128).view(np.float64)
        vf = np.ascontiguousarray(self._evecs, dtype=np.complex128).view(np.float64).reshape(-1)
        return ev, np.ascontiguousarray(self._cum, dtype=np.float64), vf

    def Print(self, with_eigensystem: bool = True) -> str:
        """The reference's ChiMatrix::Print (src/chi_matrix.cpp:129-160), returned and printed."""
        out = ["chi_matrix :\n"]
        for i in range(self.M):
            out.append("".join(_cfmt(complex(self.data[i, j])) + "\t" for j in range(self.M)) + "\n")
        if with_eigensystem and self._evals is not None:
            out.append("eigenvalues :\n" + "".join(_cfmt(complex(x)) + "\t" for x in self._evals))
            out.append("\neigenprobs :\n" + "".join(_fmt(float(x)) + "\t" for x in self._probs))
            for k in range(self.M):
                out.append(f"\neigenvector {k} :\n" + "".join(_cfmt(complex(x)) + "\t" for x in self._evecs[k]))
            out.append("\n")
        s = "".join(out)
        print(s, end="")
        return s


class CM4x4(ChiMatrix):
    """Chi matrix of a 1-qubit channel."""

    def __init__(self, data=None, *, precision: str = "DP"):
        super().__init__(4, data, precision=precision)


class CM16x16(ChiMatrix):
    """Chi matrix of a 2-qubit channel."""

    def __init__(self, data=None, *, precision: str = "DP"):
        super().__init__(16, data, precision=precision)
