"""Trotterised time evolution of an open XXZ chain, forward and adjoint, on the GPU.

    chain = XXZChain(32, J, delta=0.8, dt=0.05, steps=100, precision="SP")
    zz = chain.bond_zz(J)                 # <Z_i Z_{i+1}> for the n - 1 bonds after the evolution
    E, dE_dJ = chain.energy_and_grad(J)   # E = sum_b w_b <Z_b Z_{b+1}>, gradient w.r.t. every J_b

Each Strang step is  E(dt/2) O(dt) E(dt/2)  over the even bonds (0,1), (2,3), ... (E) and the
odd bonds (1,2), (3,4), ... (O); consecutive even half steps are merged, so 100 steps apply
E(dt/2) [O(dt) E(dt)]^99 O(dt) E(dt/2). A bond gate of duration tau is
RXX(J tau) RYY(J tau) RZZ(delta J tau) = exp(-i (J tau / 2)(XX + YY + delta ZZ)), applied as
one two-qubit gate (Apply2QubitGate, src/qureg_apply2qubitgate.cpp:14-73, semantics) and
run through the fused sweeps, which split it into phases on |00>, |11> and a 2x2 on
{|01>, |10>}. The start state is the Neel state |0101...> (qubit 1, 3, 5, ... set).

The gradient walks the circuit backwards with two registers (psi and lambda = O psi) in
fused two-vector sweeps (iqsg_adjoint_ops). With checkpoints, the forward pass keeps the
state before every `checkpoint_every`-th Strang step, and the backward pass restores psi
from the checkpoint at the end of each segment before walking it back, so rounding in the
reversed psi never builds up over more than one segment.
"""
from __future__ import annotations

import ctypes as C
import math
from typing import List, Optional, Sequence, Tuple

import numpy as np

from . import _lib
from ._lib import check, lib
from .qureg import QubitRegister


def bond_generator(delta: float) -> np.ndarray:
    """A = XX + YY + delta ZZ on (high, low) = rows 2*b(high) + b(low)."""
    a = np.zeros((4, 4), dtype=np.complex128)
    a[0, 0] = a[3, 3] = delta
    a[1, 1] = a[2, 2] = -delta
    a[1, 2] = a[2, 1] = 2.0
    return a


def bond_gate(theta: float, delta: float) -> np.ndarray:
    """exp(-i theta (XX + YY + delta ZZ)) in closed form."""
    g = np.zeros((4, 4), dtype=np.complex128)
    outer = complex(math.cos(theta * delta), -math.sin(theta * delta))
    inner = complex(math.cos(theta * delta), math.sin(theta * delta))
    c, s = math.cos(2.0 * theta), math.sin(2.0 * theta)
    g[0, 0] = g[3, 3] = outer
    g[1, 1] = g[2, 2] = inner * c
    g[1, 2] = g[2, 1] = inner * complex(0.0, -s)
    return g


def strang_layers(num_qubits: int, dt: float, steps: int) -> List[Tuple[List[int], float]]:
    """(bonds, tau) per layer in circuit order; bond b couples qubits b and b + 1."""
    even = list(range(0, num_qubits - 1, 2))
    odd = list(range(1, num_qubits - 1, 2))
    out = [(even, dt / 2)]
    for s in range(steps):
        out.append((odd, dt))
        out.append((even, dt if s < steps - 1 else dt / 2))
    return out


def _op4(kind: int, hi: int, lo: int, m: np.ndarray, value: int = 0) -> _lib.Op:
    op = _lib.Op()
    op.kind, op.t0, op.t1, op.value = kind, hi, lo, value
    a = np.ascontiguousarray(m, dtype=np.complex128).reshape(-1).view(np.float64)
    C.memmove(op.m, a.ctypes.data, a.nbytes)
    return op


class XXZChain:
    def __init__(self, num_qubits: int, J: Sequence[float], *, delta: float = 0.8, dt: float = 0.05, steps: int = 100,
                 precision: str = "SP", checkpoint_every: Optional[int] = 10, weights: Optional[Sequence[int]] = None,
                 stream: Optional[int] = None, tile_qubits: int = 0):
        self.n = int(num_qubits)
        if len(J) != self.n - 1:
            raise ValueError(f"expected {self.n - 1} couplings, got {len(J)}")
        self.J = np.asarray(J, dtype=np.float64)
        self.delta, self.dt, self.steps = float(delta), float(dt), int(steps)
        self.precision, self.stream = precision, stream
        self.checkpoint_every = checkpoint_every
        self.weights = np.ones(self.n - 1, dtype=np.int32) if weights is None else np.asarray(weights, dtype=np.int32)
        self.tile_qubits = int(tile_qubits)
        self.psi = QubitRegister(self.n, "", 0, precision=precision, stream=stream)
        self.psi.SetTileQubits(self.tile_qubits)
        self.lam: Optional[QubitRegister] = None
        self._ckpt: List[QubitRegister] = []
        self.sweeps_forward = 0
        self.sweeps_backward = 0

    # ---- circuit --------------------------------------------------------------------------
    def neel_index(self) -> int:
        return sum(1 << q for q in range(1, self.n, 2))

    def layers(self) -> List[Tuple[List[int], float]]:
        return strang_layers(self.n, self.dt, self.steps)

    def step_boundaries(self) -> List[int]:
        """Layer index at which each checkpoint segment starts (Strang steps k*C, k >= 1)."""
        C_ = self.checkpoint_every
        if not C_ or C_ >= self.steps:
            return []
        return [1 + 2 * s for s in range(C_, self.steps, C_)]

    def _pos(self, q: int) -> int:
        return self.psi.qubit_permutation.map[q]

    def _layer_ops(self, layer: Tuple[List[int], float], J: np.ndarray) -> list:
        bonds, tau = layer
        ops = []
        for b in bonds:
            g = bond_gate(0.5 * tau * J[b], self.delta)
            ops.append(_op4(_lib.OP_2Q, self._pos(b + 1), self._pos(b), g))
        return ops

    def _layer_adjoint_ops(self, layer: Tuple[List[int], float], J: np.ndarray) -> list:
        """Reverse of one layer: per bond (last first), gradient op then the inverse gate.
        G = exp(-i theta A) with theta = tau J / 2: M = 2 (d theta / d J) A = tau A."""
        bonds, tau = layer
        A = bond_generator(self.delta)
        ops = []
        for b in reversed(bonds):
            hi, lo = self._pos(b + 1), self._pos(b)
            ops.append(_op4(_lib.OP_GRAD2, hi, lo, tau * A, value=b))
            ops.append(_op4(_lib.OP_2Q, hi, lo, bond_gate(-0.5 * tau * J[b], self.delta)))
        return ops

    def _apply(self, ops: list) -> None:
        if not ops:
            return
        arr = (_lib.Op * len(ops))(*ops)
        sweeps = C.c_uint()
        check(lib.iqsg_apply_ops(self.psi._h, arr, len(arr), C.byref(sweeps)))
        self.sweeps_forward += sweeps.value

    # ---- forward ----------------------------------------------------------------------------
    def undo(self, J: Optional[Sequence[float]] = None) -> None:
        """psi <- circuit(J)^dagger psi: the layers in reverse order with every bond gate
        inverted (bonds of one layer commute)."""
        J = self.J if J is None else np.asarray(J, dtype=np.float64)
        ops = []
        for bonds, tau in reversed(self.layers()):
            ops += self._layer_ops((bonds, -tau), J)
        self._apply(ops)

    def forward(self, J: Optional[Sequence[float]] = None, keep_checkpoints: bool = False) -> None:
        """psi <- circuit(J) |Neel>; with keep_checkpoints, store the state at every
        checkpoint boundary."""
        J = self.J if J is None else np.asarray(J, dtype=np.float64)
        self.psi.Initialize("base", self.neel_index())
        bounds = set(self.step_boundaries()) if keep_checkpoints else set()
        while keep_checkpoints and len(self._ckpt) < len(bounds):
            self._ckpt.append(QubitRegister(self.n, "", 0, precision=self.precision, stream=self.stream))
        pending, k = [], 0
        for li, layer in enumerate(self.layers()):
            if li in bounds:
                self._apply(pending)
                pending = []
                check(lib.iqsg_copy(self._ckpt[k]._h, self.psi._h))
                k += 1
            pending += self._layer_ops(layer, J)
        self._apply(pending)

    def bond_zz(self, J: Optional[Sequence[float]] = None, run: bool = True) -> np.ndarray:
        """<Z_b Z_{b+1}> for every bond after the evolution."""
        if run:
            self.forward(J)
        out = np.zeros(self.n - 1)
        v = C.c_double()
        obs = (C.c_uint * 2)(3, 3)
        for b in range(self.n - 1):
            pos = (C.c_uint * 2)(self._pos(b), self._pos(b + 1))
            check(lib.iqsg_expectation_pauli(self.psi._h, 2, pos, obs, C.byref(v), None))
            out[b] = v.value
        return out

    def _edges(self):
        e = np.asarray([[self._pos(b), self._pos(b + 1)] for b in range(self.n - 1)], dtype=np.uint32).reshape(-1)
        return np.ascontiguousarray(e), np.ascontiguousarray(self.weights)

    def energy(self, J: Optional[Sequence[float]] = None) -> float:
        self.forward(J)
        e, w = self._edges()
        en = C.c_double()
        check(lib.iqsg_qaoa_observable(self.psi._h, None, self.n - 1, e.ctypes.data_as(_lib._UP),
                                       w.ctypes.data_as(_lib._IP), C.byref(en), None))
        return en.value

    # ---- adjoint --------------------------------------------------------------------------------
    def energy_and_grad(self, J: Optional[Sequence[float]] = None) -> Tuple[float, np.ndarray]:
        """E = sum_b w_b <Z_b Z_{b+1}> and dE/dJ_b for every bond, by one forward pass and one
        adjoint pass."""
        J = self.J if J is None else np.asarray(J, dtype=np.float64)
        ckpt = bool(self.step_boundaries())
        self.forward(J, keep_checkpoints=ckpt)
        if self.lam is None:
            self.lam = QubitRegister(self.n, "", 0, precision=self.precision, stream=self.stream)
        e, w = self._edges()
        en = C.c_double()
        check(lib.iqsg_qaoa_observable(self.psi._h, self.lam._h, self.n - 1, e.ctypes.data_as(_lib._UP),
                                       w.ctypes.data_as(_lib._IP), C.byref(en), None))
        grad = np.zeros(self.n - 1)
        layers = self.layers()
        starts = [0] + (self.step_boundaries() if ckpt else [])
        ends = starts[1:] + [len(layers)]
        for seg in range(len(starts) - 1, -1, -1):
            if seg < len(starts) - 1:  # psi at the end of this segment, exactly as the forward pass left it
                check(lib.iqsg_copy(self.psi._h, self._ckpt[seg]._h))
            ops = []
            for li in range(ends[seg] - 1, starts[seg] - 1, -1):
                ops += self._layer_adjoint_ops(layers[li], J)
            arr = (_lib.Op * len(ops))(*ops)
            sweeps = C.c_uint()
            check(lib.iqsg_adjoint_ops(self.psi._h, self.lam._h, arr, len(arr),
                                       grad.ctypes.data_as(_lib._DP), self.n - 1, C.byref(sweeps)))
            self.sweeps_backward += sweeps.value
        return en.value, grad

    def free_checkpoints(self) -> None:
        self._ckpt = []
