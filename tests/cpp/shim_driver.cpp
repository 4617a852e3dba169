// Drives iqs::QubitRegister<ComplexDP> from include/iqs_gb300/qureg.hpp with a text op list
// (one op per line, written by tests/test_gpu_cpp_shim.py) and writes the query results and
// the final state: the C++ drop-in header exercised exactly as a reference user would.
#include <cstdio>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "iqs_gb300/qureg.hpp"

using Reg = iqs::QubitRegister<ComplexDP>;

static TM2x2<ComplexDP> read2(std::istringstream& in) {
  TM2x2<ComplexDP> m;
  for (int r = 0; r < 2; ++r)
    for (int c = 0; c < 2; ++c) { double a, b; in >> a >> b; m(r, c) = ComplexDP(a, b); }
  return m;
}

int main(int argc, char** argv) {
  if (argc != 4) { std::fprintf(stderr, "usage: shim_driver ops.txt queries.txt state.bin\n"); return 2; }
  std::ifstream ops(argv[1]);
  std::ofstream qout(argv[2]);
  qout.precision(17);
  std::string line;
  std::getline(ops, line);
  std::istringstream head(line);
  unsigned n;
  head >> n;
  Reg psi(n, "base", 0);
  psi.EnableStatistics();
  while (std::getline(ops, line)) {
    std::istringstream in(line);
    std::string op;
    in >> op;
    unsigned a = 0, b = 0, c = 0;
    double t = 0, u = 0;
    if (op == "H") { in >> a; psi.ApplyHadamard(a); }
    else if (op == "RX") { in >> a >> t; psi.ApplyRotationX(a, t); }
    else if (op == "RY") { in >> a >> t; psi.ApplyRotationY(a, t); }
    else if (op == "RZ") { in >> a >> t; psi.ApplyRotationZ(a, t); }
    else if (op == "RXY") { in >> a >> t >> u; psi.ApplyRotationXY(a, t, u); }
    else if (op == "T") { in >> a; psi.ApplyT(a); }
    else if (op == "X") { in >> a; psi.ApplyPauliX(a); }
    else if (op == "Y") { in >> a; psi.ApplyPauliY(a); }
    else if (op == "Z") { in >> a; psi.ApplyPauliZ(a); }
    else if (op == "CNOT") { in >> a >> b; psi.ApplyCPauliX(a, b); }
    else if (op == "CZ") { in >> a >> b; psi.ApplyCPauliZ(a, b); }
    else if (op == "CPHASE") { in >> a >> b >> t; psi.ApplyCPhaseRotation(a, b, t); }
    else if (op == "CRY") { in >> a >> b >> t; psi.ApplyCRotationY(a, b, t); }
    else if (op == "SWAP") { in >> a >> b; psi.ApplySwap(a, b); }
    else if (op == "ISWAP") { in >> a >> b; psi.ApplyISwap(a, b); }
    else if (op == "TOFFOLI") { in >> a >> b >> c; psi.ApplyToffoli(a, b, c); }
    else if (op == "U1") { in >> a; psi.Apply1QubitGate(a, read2(in)); }
    else if (op == "CU1") { in >> a >> b; psi.ApplyControlled1QubitGate(a, b, read2(in)); }
    else if (op == "U2") {
      in >> a >> b;
      TM4x4<ComplexDP> m;
      for (int r = 0; r < 4; ++r)
        for (int k = 0; k < 4; ++k) { double x, y; in >> x >> y; m(r, k) = ComplexDP(x, y); }
      psi.Apply2QubitGate(a, b, m);
    } else if (op == "PERM") {
      std::vector<std::size_t> m(n);
      for (auto& x : m) in >> x;
      psi.PermuteQubits(m, "direct");
    } else if (op == "FUSION") { std::string s; in >> s; if (s == "on") psi.TurnOnFusion(); else psi.TurnOffFusion(); }
    else if (op == "PROB") { in >> a; qout << psi.GetProbability(a) << "\n"; }
    else if (op == "EXPECT") {
      unsigned k;
      in >> k;
      std::vector<unsigned> q(k), o(k);
      for (auto& x : q) in >> x;
      for (auto& x : o) in >> x;
      in >> t;
      qout << psi.ExpectationValue(q, o, t) << "\n";
    } else if (op == "NORM") { qout << psi.ComputeNorm() << "\n"; }
    else if (op == "AMP") { std::size_t i; in >> i; ComplexDP v = psi.GetGlobalAmplitude(i); qout << v.real() << " " << v.imag() << "\n"; }
    else if (!op.empty()) { std::fprintf(stderr, "unknown op %s\n", op.c_str()); return 3; }
  }
  qout << "gates " << psi.GetGateCounter()->GetTotalGateCount() << " depth " << psi.GetGateCounter()->GetParallelDepth() << "\n";
  std::vector<ComplexDP> v = psi.GetStateVector();
  std::ofstream st(argv[3], std::ios::binary);
  st.write(reinterpret_cast<const char*>(v.data()), v.size() * sizeof(ComplexDP));
  std::vector<std::size_t> map = psi.QubitMap();
  for (auto x : map) qout << "map " << x << "\n";
  return 0;
}
