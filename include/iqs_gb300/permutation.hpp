// iqs_gb300/permutation.hpp -- iqs::Permutation (include/permutation.hpp:31-408 of
// intel/intel-qs) and iqs::GateCounter (include/gate_counter.hpp:18-95), host-side classes of
// the drop-in QubitRegister, with the reference's members: the program-qubit -> data-position
// map and its inverse, index and bit-string conversions in both directions, the intermediate
// inverse maps of a local/global reorder, and gate counts with a greedy depth. Invalid
// permutations throw std::invalid_argument where the reference asserts.
#pragma once

#include <algorithm>
#include <cstdio>
#include <numeric>
#include <stdexcept>
#include <string>
#include <vector>

namespace iqs {

class Permutation {
 public:
  // map[k]: data position of element (program qubit) k; imap[p]: element at position p.
  std::vector<std::size_t> map, imap;
  std::size_t num_elements = 0;

  explicit Permutation(std::size_t n = 0) : num_elements(n) {
    std::vector<std::size_t> m(n);
    std::iota(m.begin(), m.end(), 0);
    SetNewPermutationFromMap(m, "direct");
  }
  Permutation(std::vector<std::size_t> m, std::string style_of_map = "direct") : num_elements(m.size()) {
    SetNewPermutationFromMap(m, style_of_map);
  }

  unsigned operator[](std::size_t i) const { return (unsigned)map.at(i); }
  unsigned operator[](unsigned i) const { return (unsigned)map.at(i); }
  int operator[](int i) const { return (int)map.at((std::size_t)i); }
  std::size_t size() const { return map.size(); }

  std::string GetMapStr() const { return join(map); }
  std::string GetImapStr() const { return join(imap); }

  // The element at a position (imap[position]).
  std::size_t Find(std::size_t position) const {
    for (std::size_t k = 0; k < map.size(); ++k)
      if (map[k] == position) return k;
    throw std::invalid_argument("Permutation::Find: position not in the map");
  }

  void SetNewPermutationFromMap(std::vector<std::size_t> m, std::string style_of_map = "direct") {
    if (m.size() != num_elements) throw std::invalid_argument("Permutation: map of the wrong size");
    std::vector<char> seen(m.size(), 0);
    for (auto p : m) {
      if (p >= m.size() || seen[p]) throw std::invalid_argument("Permutation: not a permutation");
      seen[p] = 1;
    }
    if (style_of_map == "direct") {
      map = m;
      imap.assign(m.size(), 0);
      for (std::size_t k = 0; k < m.size(); ++k) imap[map[k]] = k;
    } else if (style_of_map == "inverse") {
      imap = m;
      map.assign(m.size(), 0);
      for (std::size_t p = 0; p < m.size(); ++p) map[imap[p]] = p;
    } else {
      throw std::invalid_argument("Permutation: style must be \"direct\" or \"inverse\"");
    }
  }

  // Swap the positions of two elements; imap follows.
  void ExchangeTwoElements(std::size_t element_1, std::size_t element_2) {
    std::swap(map[element_1], map[element_2]);
    imap[map[element_1]] = element_1;
    imap[map[element_2]] = element_2;
  }

  // "b0 b1 b2 ..." with bit i of `in` at character i, and back.
  std::string dec2bin(std::size_t in, std::size_t num_bits) const {
    std::string s(num_bits, '0');
    for (std::size_t i = 0; i < num_bits; ++i) s[i] = ((in >> i) & 1u) ? '1' : '0';
    return s;
  }
  std::size_t bin2dec(std::string in) const {
    std::size_t v = 0;
    for (std::size_t i = 0; i < in.size(); ++i) v |= (std::size_t)(in[i] - '0') << i;
    return v;
  }

  // Index of the same basis state with program-order bits (bit k = bit map[k] of v) and back.
  std::size_t data2program_(std::size_t v) const {
    std::size_t out = 0;
    for (std::size_t k = 0; k < map.size(); ++k) out |= ((v >> map[k]) & 1u) << k;
    return out;
  }
  std::size_t program2data_(std::size_t v) const {
    std::size_t out = 0;
    for (std::size_t p = 0; p < imap.size(); ++p) out |= ((v >> imap[p]) & 1u) << p;
    return out;
  }
  // The same as bit strings (character i = bit i).
  std::string data2program(std::size_t v) const { return data2program(dec2bin(v, num_elements)); }
  std::string data2program(std::string s) const {
    std::string out(s);
    for (std::size_t k = 0; k < s.size(); ++k) out[k] = s[map[k]];
    return out;
  }
  std::string program2data(std::size_t v) const { return program2data(dec2bin(v, num_elements)); }
  std::string program2data(std::string s) const {
    std::string out(s);
    for (std::size_t p = 0; p < s.size(); ++p) out[p] = s[imap[p]];
    return out;
  }

  void Print() const { std::printf("qubit permutation: %s\n", GetMapStr().c_str()); }
  void PrintRange() const {
    for (std::size_t i = 0; i < (std::size_t(1) << num_elements); ++i)
      std::printf("map(%3lu) = %3lu\n", (unsigned long)i, (unsigned long)bin2dec(data2program(i)));
  }

  // For a reorder to target_map with positions [0, M) local: int_1_imap moves the elements that
  // end up local into their local positions (local moves only), int_2_imap then does the same
  // for the global positions; the target's imap follows.
  void ObtainIntemediateInverseMaps(std::vector<std::size_t> target_map, std::size_t M,
                                    std::vector<std::size_t>& int_1_imap, std::vector<std::size_t>& int_2_imap) const {
    if (M > num_elements || target_map.size() != num_elements)
      throw std::invalid_argument("ObtainIntemediateInverseMaps: bad sizes");
    Permutation check(target_map, "direct");  // validates target_map
    (void)check;
    int_1_imap = imap;
    for (std::size_t pos = 0; pos < M; ++pos) {
      std::size_t at = target_map[imap[pos]];
      while (at >= M) at = target_map[imap[at]];
      int_1_imap[at] = imap[pos];
    }
    int_2_imap = int_1_imap;
    for (std::size_t pos = M; pos < num_elements; ++pos) {
      std::size_t at = target_map[int_1_imap[pos]];
      while (at < M) at = target_map[int_1_imap[at]];
      int_2_imap[at] = int_1_imap[pos];
    }
  }

 private:
  static std::string join(const std::vector<std::size_t>& v) {
    std::string s;
    for (auto p : v) s += " " + std::to_string(p);
    return s;
  }
};

// Gate counts and the greedy depth (every gate one clock cycle).
class GateCounter {
 public:
  explicit GateCounter(int new_num_qubits) : num_qubits_(new_num_qubits), depth_(new_num_qubits, 0) {}

  // Resets the depth only, as the reference does.
  void Reset() { depth_.assign(num_qubits_, 0); }

  int GetTotalGateCount() const { return total_; }
  int GetOneQubitGateCount() const { return one_; }
  int GetTwoQubitGateCount() const { return two_; }
  int GetParallelDepth() const { return depth_.empty() ? 0 : *std::max_element(depth_.begin(), depth_.end()); }

  void OneQubitIncrement(int qubit) {
    ++total_;
    ++one_;
    ++depth_[qubit];
  }
  void TwoQubitIncrement(int qubit_0, int qubit_1) {
    ++total_;
    ++two_;
    const int d = std::max(depth_[qubit_0], depth_[qubit_1]) + 1;
    depth_[qubit_0] = depth_[qubit_1] = d;
  }

  void Breakdown() const {
    std::printf("The quantum circuit is composed of %d one-qubit gates and %d two-qubitgates, for a total of %d "
                "gates.\nThe greedy depth (all gates lasting one clock cycle) is %d.\n",
                GetOneQubitGateCount(), GetTwoQubitGateCount(), GetTotalGateCount(), GetParallelDepth());
  }

 private:
  int num_qubits_;
  int total_ = 0, one_ = 0, two_ = 0;
  std::vector<int> depth_;
};

}  // namespace iqs
