"""iqs_gb300: GB300 state-vector engine behind the iqs::QubitRegister API.

    import iqs_gb300 as iqs
    psi = iqs.QubitRegister(20, "base", 0)
    psi.ApplyHadamard(0)
    psi.ApplyCPauliX(0, 1)
    psi.ExpectationValueZZ(0, 1)

All state lives in GPU memory; every operation runs as a CUDA kernel in libiqsg.so.
"""
from ._lib import IqsgError, LIB_PATH, lib
from .permutation import GateCounter, Permutation
from .qureg import QubitRegister
from .adjoint import QaoaMaxCut, qaoa_energy
from .batched import BatchedAnsatz
from .rng import RandomNumberGenerator
from .chi import CM4x4, CM16x16, ChiMatrix
from .noisy import NoisyQureg, QubitRegisterMetric
from .trotter import XXZChain
from .environment import EnvFinalize, EnvFinalizeDummyRanks, EnvInit, MPIEnvironment
from .qaoa import (GetExpectationValueFromCostFunction, GetExpectationValueSquaredFromCostFunction,
                   GetHistogramFromCostFunction, GetHistogramFromCostFunctionWithWeightsBinned,
                   GetHistogramFromCostFunctionWithWeightsRounded, ImplementQaoaLayerBasedOnCostFunction,
                   InitializeVectorAsMaxCutCostFunction, InitializeVectorAsWeightedMaxCutCostFunction)

__all__ = [
    "QubitRegister", "Permutation", "GateCounter", "IqsgError", "LIB_PATH", "lib",
    "InitializeVectorAsMaxCutCostFunction", "ImplementQaoaLayerBasedOnCostFunction",
    "GetExpectationValueFromCostFunction", "GetExpectationValueSquaredFromCostFunction",
    "InitializeVectorAsWeightedMaxCutCostFunction", "GetHistogramFromCostFunction",
    "GetHistogramFromCostFunctionWithWeightsRounded", "GetHistogramFromCostFunctionWithWeightsBinned",
    "QaoaMaxCut", "qaoa_energy", "BatchedAnsatz", "XXZChain", "RandomNumberGenerator", "ChiMatrix", "CM4x4", "CM16x16", "NoisyQureg", "QubitRegisterMetric",
    "EnvInit", "EnvFinalize", "EnvFinalizeDummyRanks", "MPIEnvironment",
]
