"""Batches of small circuits of different sizes: forward energies and adjoint gradients of a
hardware-efficient ansatz for every instance in one persistent launch, replayed as a CUDA graph.

    b = BatchedAnsatz([(n_i, L_i, [(coeff, "XIZY..."), ...]), ...], precision="SP")
    energies = b.run(params)                          # params: flat, see param_slices()
    energies, grads = b.run(params, with_grad=True)
    b.autotune(params)                                # picks threads/CTA and CTAs/SM

Instance i: from |0..0>, L_i layers of RZ(phi_q) then RY(theta_q) on every qubit q, then
CZ(q, q+1) for q = 0..n-2. Pauli strings are written qubit 0 first ("XZ" = X on qubit 0,
Z on qubit 1).
"""
from __future__ import annotations

import ctypes as C
import time
from typing import List, Optional, Sequence, Tuple

import numpy as np

from . import _lib
from ._lib import check, lib

_PREC = {"DP": _lib.COMPLEX_DP, "SP": _lib.COMPLEX_SP}


def pauli_term(coeff: float, letters: str) -> "_lib.PauliTerm":
    t = _lib.PauliTerm()
    xm = zm = ny = 0
    for q, ch in enumerate(letters):
        b = 1 << q
        if ch == "X":
            xm |= b
        elif ch == "Y":
            xm |= b
            zm |= b
            ny += 1
        elif ch == "Z":
            zm |= b
        elif ch != "I":
            raise ValueError(f"Pauli letter {ch!r} not in IXYZ")
    t.xmask, t.zmask, t.ny, t.coeff = xm, zm, ny % 4, float(coeff)
    return t


class BatchedAnsatz:
    def __init__(self, instances: Sequence[Tuple[int, int, Sequence[Tuple[float, str]]]], *, precision: str = "SP",
                 stream: Optional[int] = None):
        self.instances = [(int(n), int(L), list(terms)) for n, L, terms in instances]
        nq = np.asarray([n for n, _, _ in self.instances], dtype=np.uint32)
        nl = np.asarray([L for _, L, _ in self.instances], dtype=np.uint32)
        nt = np.asarray([len(t) for _, _, t in self.instances], dtype=np.uint32)
        flat = [pauli_term(c, s) for _, _, terms in self.instances for c, s in terms]
        arr = (_lib.PauliTerm * max(1, len(flat)))(*flat)
        self._h = C.c_void_p()
        check(lib.iqsg_batch_create(len(self.instances), nq.ctypes.data_as(_lib._UP), nl.ctypes.data_as(_lib._UP),
                                    nt.ctypes.data_as(_lib._UP), arr, _PREC[precision], C.c_void_p(stream or 0),
                                    C.byref(self._h)))
        npar, namps = C.c_uint64(), C.c_uint64()
        check(lib.iqsg_batch_info(self._h, C.byref(npar), C.byref(namps)))
        self.num_params, self.total_amplitudes = npar.value, namps.value
        offs = np.cumsum([0] + [2 * n * L for n, L, _ in self.instances])
        self._slices = [slice(int(offs[i]), int(offs[i + 1])) for i in range(len(self.instances))]
        self.launch = (512, 2)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            lib.iqsg_batch_destroy(h)
            self._h = C.c_void_p()

    def param_slices(self) -> List[slice]:
        """Slice of the flat parameter vector of each instance ([layer][qubit][phi, theta])."""
        return list(self._slices)

    def set_launch(self, threads: int, ctas_per_sm: int) -> None:
        check(lib.iqsg_batch_set_launch(self._h, int(threads), int(ctas_per_sm)))
        self.launch = (int(threads), int(ctas_per_sm))

    def run(self, params, with_grad: bool = False):
        p = np.ascontiguousarray(np.asarray(params, dtype=np.float64))
        if p.size != self.num_params:
            raise ValueError(f"expected {self.num_params} parameters, got {p.size}")
        e = np.empty(len(self.instances))
        g = np.empty(self.num_params) if with_grad else None
        check(lib.iqsg_batch_run(self._h, p.ctypes.data_as(_lib._DP), 1 if with_grad else 0,
                                 e.ctypes.data_as(_lib._DP), g.ctypes.data_as(_lib._DP) if with_grad else None))
        return (e, g) if with_grad else e

    def autotune(self, params, with_grad: bool = True,
                 shapes=((128, 4), (128, 8), (256, 2), (256, 4), (512, 1), (512, 2)), trials: int = 2):
        """Time every (threads per CTA, CTAs per SM) and keep the fastest; returns the table."""
        table = []
        for th, cps in shapes:
            self.set_launch(th, cps)
            self.run(params, with_grad)  # records the graph
            best = float("inf")
            for _ in range(trials):
                t0 = time.perf_counter()
                self.run(params, with_grad)
                best = min(best, time.perf_counter() - t0)
            table.append((th, cps, best))
        th, cps, _ = min(table, key=lambda r: r[2])
        self.set_launch(th, cps)
        self.run(params, with_grad)
        return table
