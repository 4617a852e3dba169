"""QAOA MaxCut energies and adjoint-mode gradients on the GPU, with a torch.autograd.Function.

    circ = QaoaMaxCut(n, edges)                      # edges: [(u, v), ...] program qubits
    E = circ.energy(gammas, betas)                   # forward only
    E, dg, db = circ.energy_and_grad(gammas, betas)  # one forward + one adjoint backward
    E_t = qaoa_energy(params_tensor, circ)           # torch: params = [gammas..., betas...]

Circuit (per layer l): exp(-i gamma_l H_C) with H_C = 1/2 sum_e w_e Z_u Z_v, then RX(2 beta_l)
on every qubit, from |+>^n; energy E = sum_e w_e <Z_u Z_v>. The cost layer equals the
reference's ImplementQaoaLayerBasedOnCostFunction with the MaxCut cost vector
(src/qaoa_features.cpp:248-264) up to a global phase; the mixer is ApplyRotationX(q, 2 beta).
The backward pass keeps two state vectors (psi and lambda = O psi) and walks the layers in
reverse; a third vector is never needed.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional, Sequence, Tuple

import numpy as np

from ._lib import check, iptr, lib, uptr
from .qureg import QubitRegister


class QaoaMaxCut:
    def __init__(self, num_qubits: int, edges: Sequence[Tuple[int, int]], weights: Optional[Sequence[int]] = None,
                 *, precision: str = "DP", stream: Optional[int] = None, checkpoint: bool = False):
        """checkpoint=True keeps the state after the cost phase and after the mixer of every
        layer (2p extra vectors) so the backward pass walks only lambda back: fewer
        operations per gradient, more memory."""
        self.n = int(num_qubits)
        self.edges = [(int(u), int(v)) for u, v in edges]
        self.weights = None if weights is None else [int(w) for w in weights]
        self.psi = QubitRegister(self.n, "", 0, precision=precision, stream=stream)
        self.lam: Optional[QubitRegister] = None
        self._edge_arr = np.ascontiguousarray(np.asarray(self.edges, dtype=np.uint32).reshape(-1))
        self._w_arr = None if self.weights is None else np.ascontiguousarray(np.asarray(self.weights, dtype=np.int32))
        self.precision = precision
        self.stream = stream
        self._prepared = None  # parameters psi currently holds the circuit state of
        self.checkpoint = checkpoint
        self._ckpt = []

    def _ew(self):
        pos = np.asarray([self.psi.qubit_permutation.map[q] for q in self._edge_arr], dtype=np.uint32)
        return len(self.edges), uptr(pos), (iptr(self._w_arr) if self._w_arr is not None else None), pos

    def prepare(self, gammas: Sequence[float], betas: Sequence[float]) -> None:
        """psi <- circuit(gammas, betas) |+>^n."""
        if len(gammas) != len(betas):
            raise ValueError("gammas and betas differ in length")
        self.psi.Initialize("++++", 0)
        ne, e, w, _keep = self._ew()
        for g, b in zip(gammas, betas):
            check(lib.iqsg_qaoa_layer(self.psi._h, ne, e, w, float(g), float(b)))
        self._prepared = np.concatenate([np.asarray(gammas, float), np.asarray(betas, float)])

    def _observable(self, with_lambda: bool) -> float:
        ne, e, w, _keep = self._ew()
        if with_lambda and self.lam is None:
            self.lam = QubitRegister(self.n, "", 0, precision=self.precision, stream=self.stream)
        en, n2 = C.c_double(), C.c_double()
        check(lib.iqsg_qaoa_observable(self.psi._h, self.lam._h if with_lambda else None, ne, e, w,
                                       C.byref(en), C.byref(n2)))
        return en.value

    def energy(self, gammas: Sequence[float], betas: Sequence[float]) -> float:
        self.prepare(gammas, betas)
        return self._observable(False)

    def _grad_checkpointed(self, gammas, betas):
        p = len(gammas)
        while len(self._ckpt) < 2 * p:
            self._ckpt.append(QubitRegister(self.n, "", 0, precision=self.precision, stream=self.stream))
        self.psi.Initialize("++++", 0)
        ne, ep, w, _keep = self._ew()
        for l in range(p):
            check(lib.iqsg_qaoa_layer_ckpt(self.psi._h, self._ckpt[2 * l]._h, self._ckpt[2 * l + 1]._h, ne, ep, w,
                                           float(gammas[l]), float(betas[l])))
        self._prepared = np.concatenate([np.asarray(gammas, float), np.asarray(betas, float)])
        e = self._observable(True)
        dg, db = np.zeros(p), np.zeros(p)
        gg, gb = C.c_double(), C.c_double()
        for l in range(p - 1, -1, -1):
            check(lib.iqsg_qaoa_layer_backward_ckpt(self.lam._h, self._ckpt[2 * l]._h, self._ckpt[2 * l + 1]._h, ne, ep,
                                                    w, float(gammas[l]), float(betas[l]), C.byref(gg), C.byref(gb)))
            dg[l], db[l] = gg.value, gb.value
        return e, dg, db

    def energy_and_grad(self, gammas: Sequence[float], betas: Sequence[float]):
        """Energy and its gradient by the adjoint method: (E, dE/dgamma[p], dE/dbeta[p]).
        The forward circuit is skipped when psi already holds the state of these parameters."""
        if self.checkpoint:
            return self._grad_checkpointed(gammas, betas)
        want = np.concatenate([np.asarray(gammas, float), np.asarray(betas, float)])
        if self._prepared is None or not np.array_equal(self._prepared, want):
            self.prepare(gammas, betas)
        self._prepared = None  # the backward sweep walks psi back to |+>^n
        e = self._observable(True)
        ne, ep, w, _keep = self._ew()
        p = len(gammas)
        dg, db = np.zeros(p), np.zeros(p)
        gg, gb = C.c_double(), C.c_double()
        for l in range(p - 1, -1, -1):
            check(lib.iqsg_qaoa_layer_backward(self.psi._h, self.lam._h, ne, ep, w, float(gammas[l]), float(betas[l]),
                                               C.byref(gg), C.byref(gb)))
            dg[l], db[l] = gg.value, gb.value
        return e, dg, db

    def finite_difference_grad(self, gammas: Sequence[float], betas: Sequence[float], h: float = 1e-6):
        """Central differences, two forward circuits per parameter."""
        g0, b0 = np.asarray(gammas, float), np.asarray(betas, float)
        dg, db = np.zeros_like(g0), np.zeros_like(b0)
        for k in range(len(g0)):
            gp, gm = g0.copy(), g0.copy()
            gp[k] += h
            gm[k] -= h
            dg[k] = (self.energy(gp, b0) - self.energy(gm, b0)) / (2 * h)
            bp, bm = b0.copy(), b0.copy()
            bp[k] += h
            bm[k] -= h
            db[k] = (self.energy(g0, bp) - self.energy(g0, bm)) / (2 * h)
        return dg, db


def qaoa_energy(params, circuit: QaoaMaxCut):
    """Differentiable energy: params = torch tensor [gamma_1..gamma_p, beta_1..beta_p] (CPU or
    CUDA, any float dtype); returns a 0-d tensor. Forward prepares the state and measures the
    energy; backward runs the adjoint kernels from that state (re-preparing it first if the
    circuit object was used for other parameters in between)."""
    import torch

    class _QaoaEnergy(torch.autograd.Function):
        @staticmethod
        def forward(ctx, prm):
            v = prm.detach().to("cpu", torch.float64).numpy().copy()
            p = v.size // 2
            e = circuit.energy(v[:p], v[p:])
            ctx.params = v
            ctx.device, ctx.dtype = prm.device, prm.dtype
            return torch.tensor(e, dtype=prm.dtype, device=prm.device)

        @staticmethod
        def backward(ctx, grad_out):
            v = ctx.params
            p = v.size // 2
            _e, dg, db = circuit.energy_and_grad(v[:p], v[p:])
            g = torch.from_numpy(np.concatenate([dg, db])).to(ctx.device, ctx.dtype)
            return grad_out * g

    return _QaoaEnergy.apply(params)
