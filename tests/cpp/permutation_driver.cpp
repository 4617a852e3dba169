// The reference's Permutation and GateCounter unit tests (unit_test/include/permutation_test.hpp,
// unit_test/include/gate_counter_test.hpp) against the drop-in header. Host code only; exits
// non-zero on the first failed check.
#include <cmath>
#include <cstdio>
#include <vector>

#include "iqs_gb300/qureg.hpp"

static int failures = 0;
#define CHECK(c)                                                   \
  do {                                                             \
    if (!(c)) {                                                    \
      std::fprintf(stderr, "%s:%d: %s\n", __FILE__, __LINE__, #c); \
      ++failures;                                                  \
    }                                                              \
  } while (0)

using V = std::vector<std::size_t>;

int main() {
  {  // InitializationToIdentitylPermutation
    iqs::Permutation p(6);
    CHECK(p.num_elements == 6);
    for (unsigned i = 0; i < 6; ++i) CHECK(p[i] == i && p.imap[i] == i);
  }
  {  // BasicUse
    iqs::Permutation p(6);
    V map = {1, 2, 0, 3, 5, 4}, imap = {2, 0, 1, 3, 5, 4};
    p.SetNewPermutationFromMap(map, "direct");
    for (unsigned i = 0; i < 6; ++i) CHECK(p[i] == map[i] && p.imap[map[i]] == i && p.imap[i] == imap[i]);
    p.SetNewPermutationFromMap(map, "inverse");
    for (unsigned i = 0; i < 6; ++i) CHECK(p.imap[i] == map[i] && p.map[i] == imap[i]);
  }
  {  // ExchangeTwoElements
    iqs::Permutation p(6);
    V map = {1, 2, 0, 3, 5, 4};
    p.SetNewPermutationFromMap(map, "direct");
    unsigned e1 = 2, e2 = 4, p1 = p[e1], p2 = p[e2];
    p.ExchangeTwoElements(e1, e2);
    map[e1] = p2;
    map[e2] = p1;
    for (unsigned i = 0; i < 6; ++i) CHECK(p[i] == map[i]);
    e1 = 4;
    e2 = 0;
    p1 = map[e1];
    p2 = map[e2];
    map[e1] = p2;
    map[e2] = p1;
    p.ExchangeTwoElements(e1, e2);
    for (unsigned i = 0; i < 6; ++i) CHECK(p[i] == map[i] && p.imap[map[i]] == i);
  }
  {  // Program2Data
    iqs::Permutation p(3);
    for (std::size_t v = 0; v < 8; ++v) CHECK(p.program2data_(v) == v);
    p.SetNewPermutationFromMap({1, 0, 2}, "direct");
    V want = {0, 2, 1, 3, 4, 6, 5, 7};
    for (std::size_t v = 0; v < 8; ++v) CHECK(p.program2data_(v) == want[v] && p.data2program_(v) == p.program2data_(v));
    p.SetNewPermutationFromMap({1, 2, 0}, "direct");
    want = {0, 2, 4, 6, 1, 3, 5, 7};
    for (std::size_t v = 0; v < 8; ++v) CHECK(p.program2data_(v) == want[v]);
  }
  {  // Data2Program
    iqs::Permutation p(4);
    for (std::size_t v = 0; v < 16; ++v) CHECK(p.data2program_(v) == v);
    p.SetNewPermutationFromMap({2, 3, 1, 0}, "inverse");
    V want = {0, 4, 8, 12, 2, 6, 10, 14, 1, 5, 9, 13, 3, 7, 11, 15};
    for (std::size_t v = 0; v < 16; ++v) {
      CHECK(p.data2program_(v) == want[v]);
      CHECK(p.bin2dec(p.data2program(v)) == want[v]);   // the bit-string forms agree
      CHECK(p.program2data_(p.data2program_(v)) == v);
      CHECK(p.program2data(p.data2program(v)) == p.dec2bin(v, 4));
    }
  }
  {  // ObtainIntemediateInverseMaps
    iqs::Permutation p(V{0, 1, 2, 3, 4, 5, 6, 7}, "direct");
    V i1, i2;
    p.ObtainIntemediateInverseMaps({1, 5, 2, 3, 6, 0, 7, 4}, 5, i1, i2);
    CHECK((i1 == V{1, 0, 2, 3, 4, 5, 6, 7}) && (i2 == V{1, 0, 2, 3, 4, 5, 7, 6}));
    p.SetNewPermutationFromMap({1, 5, 2, 3, 6, 0, 7, 4}, "direct");
    p.ObtainIntemediateInverseMaps({1, 6, 7, 4, 3, 2, 0, 5}, 5, i1, i2);
    CHECK((i1 == V{2, 0, 5, 7, 3, 1, 4, 6}) && (i2 == V{2, 0, 5, 7, 3, 4, 1, 6}));
  }
  {  // Find, strings, invalid input
    iqs::Permutation p(V{2, 0, 1});
    CHECK(p.Find(0) == 1 && p.Find(2) == 0);
    CHECK(p.GetMapStr() == " 2 0 1" && p.GetImapStr() == " 1 2 0");
    bool threw = false;
    try {
      p.SetNewPermutationFromMap({0, 0, 1});
    } catch (const std::invalid_argument&) {
      threw = true;
    }
    CHECK(threw);
  }
  {  // GateCounter
    iqs::GateCounter g(4);
    g.OneQubitIncrement(0);
    g.OneQubitIncrement(0);
    g.TwoQubitIncrement(0, 3);
    g.OneQubitIncrement(2);
    CHECK(g.GetOneQubitGateCount() == 3 && g.GetTwoQubitGateCount() == 1 && g.GetTotalGateCount() == 4);
    CHECK(g.GetParallelDepth() == 3);
    g.Reset();
    CHECK(g.GetParallelDepth() == 0 && g.GetTotalGateCount() == 4);
  }
  {  // conversion_test.hpp BasicUse and the bit utilities
    CHECK(iqs::toString(1) == "1" && iqs::toString('a') == "a" && iqs::toString(std::string("s")) == "s");
    CHECK(iqs::floor_power_of_two(5u) == 4 && iqs::floor_power_of_two(8u) == 8 && iqs::floor_power_of_two(1u) == 1);
    CHECK(iqs::ilog2(std::size_t(1) << 33) == 33 && iqs::isPowerOf2(64) && !iqs::isPowerOf2(12) && !iqs::isPowerOf2(0));
    CHECK(iqs::highestBit(0x90u) == 7 && iqs::popcnt(uint64_t(0xF0F0)) == 8 && UL(3) == std::size_t(3));
  }
  {  // the one-state pool environment
    iqs::mpi::Environment::Init();
    CHECK(iqs::mpi::Environment::GetSharedInstance() != nullptr && iqs::mpi::Environment::IsUsefulRank());
    CHECK(iqs::mpi::Environment::GetStateSize() == 1 && iqs::mpi::Environment::GetNumStates() == 1);
    CHECK(iqs::mpi::Environment::IncoherentSumOverAllStatesOfPool<double>(0.5) == 0.5);
    iqs::mpi::StateBarrier();
    iqs::mpi::Environment::Finalize();
    CHECK(iqs::mpi::Environment::GetSharedInstance() == nullptr);
  }
  std::printf("%d failures\n", failures);
  return failures ? 1 : 0;
}
