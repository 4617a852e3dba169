"""QAOA helpers over GPU registers (include/qaoa_features.hpp, src/qaoa_features.cpp).

The cost "vector" is a QubitRegister whose real parts hold the cost of each basis state,
exactly as in the reference. Names and argument order follow iqs::qaoa.
"""
from __future__ import annotations

import ctypes as C
from typing import Sequence

import numpy as np

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
