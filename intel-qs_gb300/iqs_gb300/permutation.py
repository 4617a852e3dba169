"""Host-side qubit order: program qubit <-> data position (include/permutation.hpp)."""
from __future__ import annotations

from typing import Iterable, List


class Permutation:
    """Program-qubit -> data-position map, as iqs::Permutation (include/permutation.hpp:31-408).

    ``map[q]`` is the position of program qubit q, ``imap[p]`` the program qubit stored at
    position p. Bit p of a data index is position p.
    """

    def __init__(self, m, style_of_map: str = "direct"):
        if isinstance(m, int):
            m = list(range(m))
        self.map: List[int] = []
        self.imap: List[int] = []
        self.SetNewPermutationFromMap(list(m), style_of_map)

    @property
    def num_elements(self) -> int:
        return len(self.map)

    def __getitem__(self, q: int) -> int:
        if not 0 <= q < len(self.map):
            raise IndexError(f"qubit {q} out of range for {len(self.map)} qubits")
        return self.map[q]

    def __len__(self) -> int:
        return len(self.map)

    def __eq__(self, other) -> bool:
        return isinstance(other, Permutation) and self.map == other.map

    def SetNewPermutationFromMap(self, m: List[int], style_of_map: str = "direct") -> None:
        """include/permutation.hpp:157-185; raises ValueError where the reference asserts."""
        n = len(m)
        if sorted(m) != list(range(n)):
            raise ValueError(f"not a permutation of 0..{n - 1}: {m}")
        if style_of_map == "direct":
            self.map = list(m)
            self.imap = [0] * n
            for q, p in enumerate(self.map):
                self.imap[p] = q
        elif style_of_map == "inverse":
            self.imap = list(m)
            self.map = [0] * n
            for p, q in enumerate(self.imap):
                self.map[q] = p
        else:
            raise ValueError(f"style_of_map must be 'direct' or 'inverse', not {style_of_map!r}")

    def ExchangeTwoElements(self, e1: int, e2: int) -> None:
        """include/permutation.hpp:193-201."""
        p1, p2 = self.map[e1], self.map[e2]
        self.map[e1], self.map[e2] = p2, p1
        self.imap[p1], self.imap[p2] = e2, e1

    def Find(self, position: int) -> int:
        return self.imap[position]

    def data2program_(self, v: int) -> int:
        """Bit q of the result = bit map[q] of v (include/permutation.hpp:249-255)."""
        out = 0
        for q, p in enumerate(self.map):
            out |= ((v >> p) & 1) << q
        return out

    def program2data_(self, v: int) -> int:
        """Bit p of the result = bit imap[p] of v (include/permutation.hpp:258-264)."""
        out = 0
        for p, q in enumerate(self.imap):
            out |= ((v >> q) & 1) << p
        return out

    @staticmethod
    def dec2bin(v: int, num_bits: int) -> str:
        """Bits of v, least significant first (include/permutation.hpp:208-218)."""
        return "".join("1" if (v >> i) & 1 else "0" for i in range(num_bits))

    @staticmethod
    def bin2dec(s: str) -> int:
        """Inverse of dec2bin: character i is bit i (include/permutation.hpp:223-229)."""
        return sum(1 << i for i, c in enumerate(s) if c == "1")

    def data2program(self, v) -> str:
        """Program-order bit string of a data index (or of a data bit string): character q is
        bit map[q] (include/permutation.hpp:267-292)."""
        s = v if isinstance(v, str) else self.dec2bin(int(v), len(self.map))
        return "".join(s[p] for p in self.map)

    def program2data(self, v) -> str:
        """Data-order bit string of a program index (or program bit string): character p is
        bit imap[p] (include/permutation.hpp:295-306)."""
        s = v if isinstance(v, str) else self.dec2bin(int(v), len(self.map))
        return "".join(s[q] for q in self.imap)

    def Print(self) -> str:
        line = f"qubit permutation: {self.GetMapStr()}"
        print(line)
        return line

    def PrintRange(self) -> str:
        lines = [f"map({i:3d}) = {self.bin2dec(self.data2program(i)):3d}" for i in range(1 << len(self.map))]
        print("\n".join(lines))
        return "\n".join(lines)

    def ObtainIntemediateInverseMaps(self, target_map: List[int], M: int):
        """For a reorder to target_map with positions [0, M) local, the inverse maps after the
        local-only moves and after the global-only moves (include/permutation.hpp:345-380)."""
        n = len(self.map)
        if M > n or sorted(target_map) != list(range(n)):
            raise ValueError("ObtainIntemediateInverseMaps: target_map must be a permutation and M <= n")
        int_1 = list(self.imap)
        for pos in range(M):
            at = target_map[self.imap[pos]]
            while at >= M:
                at = target_map[self.imap[at]]
            int_1[at] = self.imap[pos]
        int_2 = list(int_1)
        for pos in range(M, n):
            at = target_map[int_1[pos]]
            while at < M:
                at = target_map[int_1[at]]
            int_2[at] = int_1[pos]
        return int_1, int_2

    def GetMapStr(self) -> str:
        return "".join(f" {p}" for p in self.map)

    def GetImapStr(self) -> str:
        return "".join(f" {q}" for q in self.imap)

    def copy(self) -> "Permutation":
        return Permutation(self.map, "direct")


class GateCounter:
    """One/two-qubit gate counts and greedy depth (include/gate_counter.hpp:18-95)."""

    def __init__(self, num_qubits: int):
        self.num_qubits = num_qubits
        self.total_gate_count = 0
        self.one_qubit_gate_count = 0
        self.two_qubit_gate_count = 0
        self.parallel_depth = [0] * num_qubits

    def Reset(self) -> None:
        self.parallel_depth = [0] * self.num_qubits

    def GetTotalGateCount(self) -> int:
        return self.total_gate_count

    def GetOneQubitGateCount(self) -> int:
        return self.one_qubit_gate_count

    def GetTwoQubitGateCount(self) -> int:
        return self.two_qubit_gate_count

    def GetParallelDepth(self) -> int:
        return max(self.parallel_depth) if self.parallel_depth else 0

    def OneQubitIncrement(self, q: int) -> None:
        self.total_gate_count += 1
        self.one_qubit_gate_count += 1
        self.parallel_depth[q] += 1

    def TwoQubitIncrement(self, q0: int, q1: int) -> None:
        self.total_gate_count += 1
        self.two_qubit_gate_count += 1
        d = max(self.parallel_depth[q0], self.parallel_depth[q1]) + 1
        self.parallel_depth[q0] = d
        self.parallel_depth[q1] = d

    def Breakdown(self) -> str:
        s = (f"The quantum circuit is composed of {self.one_qubit_gate_count} one-qubit gates and "
             f"{self.two_qubit_gate_count} two-qubitgates, for a total of {self.total_gate_count} gates.\n"
             f"The greedy depth (all gates lasting one clock cycle) is {self.GetParallelDepth()}.\n")
        print(s, end="")
        return s


def check_distinct(qubits: Iterable[int], n: int, what: str) -> None:
    seen = set()
    for q in qubits:
        if not 0 <= q < n:
            raise ValueError(f"{what}: qubit {q} out of range for {n} qubits")
        if q in seen:
            raise ValueError(f"{what}: qubit {q} repeated")
        seen.add(q)
