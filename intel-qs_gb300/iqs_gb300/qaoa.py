"""QAOA helpers over GPU registers (include/qaoa_features.hpp, src/qaoa_features.cpp).

The cost "vector" is a QubitRegister whose real parts hold the cost of each basis state,
exactly as in the reference. Names and argument order follow iqs::qaoa.
"""
from __future__ import annotations

import ctypes as C
from typing import Sequence

import numpy as np

from . import _lib
from ._lib import check, iptr, lib, uptr
from .qureg import QubitRegister


def InitializeVectorAsMaxCutCostFunction(diag: QubitRegister, adjacency: Sequence[int]) -> int:
    """diag[i] = (number of cut edges of basis state d2p(i), 0); returns the maximum cut
    (src/qaoa_features.cpp:73-143). adjacency: n*n ints, symmetric, zero diagonal."""
    n = diag.NumQubits()
    adj = np.ascontiguousarray(np.asarray(adjacency, dtype=np.int32).reshape(-1))
    if adj.size != n * n:
        raise ValueError(f"adjacency must have {n * n} entries, got {adj.size}")
    mp = np.asarray(diag.qubit_permutation.map, dtype=np.uint32)
    diag._flush()
    mx = C.c_int()
    check(lib.iqsg_maxcut_cost(diag._h, iptr(adj), uptr(mp), C.byref(mx)))
    return mx.value


def InitializeVectorAsWeightedMaxCutCostFunction(diag: QubitRegister, adjacency: Sequence[float]) -> float:
    """diag[i] = (total weight of the edges cut by basis state d2p(i), 0); returns the maximum
    (src/qaoa_features.cpp:153-239). adjacency: n*n weights, symmetric, zero diagonal."""
    n = diag.NumQubits()
    adj = np.ascontiguousarray(np.asarray(adjacency, dtype=np.float64).reshape(-1))
    if adj.size != n * n:
        raise ValueError(f"adjacency must have {n * n} entries, got {adj.size}")
    if diag.precision == "SP":  # the reference's BaseType adjacency
        adj = adj.astype(np.float32).astype(np.float64)
    mp = np.asarray(diag.qubit_permutation.map, dtype=np.uint32)
    diag._flush()
    mx = C.c_double()
    check(lib.iqsg_weighted_maxcut_cost(diag._h, adj.ctypes.data_as(_lib._DP), uptr(mp), C.byref(mx)))
    return mx.value


def _histogram(psi: QubitRegister, diag: QubitRegister, mode: int, max_value: float, bin_width: float,
               num_bins: int) -> list:
    if psi.qubit_permutation.map != diag.qubit_permutation.map:
        raise ValueError("psi and diag have different qubit orders")
    if num_bins <= 0:
        raise ValueError("max_value must be positive")
    psi._flush()
    diag._flush()
    out = np.zeros(num_bins)
    check(lib.iqsg_cost_histogram(psi._h, diag._h, mode, float(max_value), float(bin_width),
                                  out.ctypes.data_as(_lib._DP), num_bins))
    return [float(x) for x in out]


def GetHistogramFromCostFunction(psi: QubitRegister, diag: QubitRegister, max_value: int) -> list:
    """Probability of each integer cost value 0..max_value (src/qaoa_features.cpp:335-400)."""
    if int(max_value) != max_value or max_value <= 0:
        raise ValueError("max_value must be a positive integer")
    return _histogram(psi, diag, _lib.HIST_INTEGER, max_value, 1.0, int(max_value) + 1)


def GetHistogramFromCostFunctionWithWeightsRounded(psi: QubitRegister, diag: QubitRegister, max_value: float) -> list:
    """Probability of floor(cost + 1e-7) for each bin 0..floor(max_value)
    (src/qaoa_features.cpp:402-469)."""
    return _histogram(psi, diag, _lib.HIST_ROUNDED, max_value, 1.0, int(np.floor(max_value)) + 1)


def GetHistogramFromCostFunctionWithWeightsBinned(psi: QubitRegister, diag: QubitRegister, max_value: float,
                                                  bin_width: float) -> list:
    """Probability of floor(cost / bin_width + 1e-7) for each bin 0..ceil(max_value / bin_width)
    (src/qaoa_features.cpp:471-538)."""
    if not bin_width > 0:
        raise ValueError("bin_width must be positive")
    return _histogram(psi, diag, _lib.HIST_BINNED, max_value, bin_width, int(np.ceil(max_value / bin_width)) + 1)


def ImplementQaoaLayerBasedOnCostFunction(psi: QubitRegister, diag: QubitRegister, gamma: float) -> None:
    """psi[i] *= exp(-i gamma Re diag[i]) (src/qaoa_features.cpp:248-264)."""
    if psi.qubit_permutation.map != diag.qubit_permutation.map:
        raise ValueError("psi and diag have different qubit orders")
    psi._flush()
    diag._flush()
    check(lib.iqsg_apply_cost_phase(psi._h, diag._h, psi._bt(gamma)))


def GetExpectationValueFromCostFunction(psi: QubitRegister, diag: QubitRegister) -> float:
    """sum_i Re diag[i] |psi_i|^2 (src/qaoa_features.cpp:273-300)."""
    if psi.qubit_permutation.map != diag.qubit_permutation.map:
        raise ValueError("psi and diag have different qubit orders")
    psi._flush()
    diag._flush()
    v = C.c_double()
    check(lib.iqsg_cost_expectation(psi._h, diag._h, 1, C.byref(v)))
    return v.value


def GetExpectationValueSquaredFromCostFunction(psi: QubitRegister, diag: QubitRegister) -> float:
    """sum_i (Re diag[i])^2 |psi_i|^2 (src/qaoa_features.cpp:304-331)."""
    if psi.qubit_permutation.map != diag.qubit_permutation.map:
        raise ValueError("psi and diag have different qubit orders")
    psi._flush()
    diag._flush()
    v = C.c_double()
    check(lib.iqsg_cost_expectation(psi._h, diag._h, 2, C.byref(v)))
    return v.value
