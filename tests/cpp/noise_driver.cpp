// A caller of the noise API of the C++ drop-in header (iqs::RandomNumberGenerator, ChiMatrix,
// QubitRegister::ApplyNoiseGate / ApplyChannel, NoisyQureg), written as against the reference.
// Reads a case from standard input, prints results with 17 significant digits.
//
//   noise_driver rng      : "prec seed nops" + nops lines "kind n stream"  (no GPU needed)
//   noise_driver eigen    : 2x2 chi [[1,3],[3,7]] -> eigenvalues and eigenvectors (no GPU)
//   noise_driver noise    : "prec n seed T1 T2 steps" + 2^n "re im" + steps "qubit duration"
//   noise_driver noisy    : "prec n seed T1 T2 Ts Td nprog" + nprog "kind a b angle m(8)"
//   noise_driver channel  : "prec n seed M steps" + M "re im" + M*M "re im" + 2^n "re im" + qubits
// prec is 0 for ComplexDP, 1 for ComplexSP.
#include <cstdio>
#include <iostream>
#include <string>
#include <vector>

#include "iqs_gb300/qureg.hpp"

namespace {

const char* kStreams[3] = {"pool", "state", "local"};

template <class B>
void run_rng(std::size_t seed, int nops) {
  auto* rng = new iqs::RandomNumberGenerator<B>();
  rng->SetSeedStreamPtrs(seed);
  for (int i = 0; i < nops; ++i) {
    int kind, n, st;
    std::cin >> kind >> n >> st;
    std::vector<B> v(n > 0 ? n : 1);
    std::vector<int> iv(n > 0 ? n : 1);
    if (kind == 0) rng->UniformRandomNumbers(v.data(), n, 0, 1, kStreams[st]);
    if (kind == 1) rng->UniformRandomNumbers(v.data(), n, -2, 5, kStreams[st]);
    if (kind == 2) rng->GaussianRandomNumbers(v.data(), n, kStreams[st]);
    if (kind == 3) {
      rng->RandomIntegersInRange(iv.data(), n, -3, 17, kStreams[st]);
      for (int j = 0; j < n; ++j) v[j] = (B)iv[j];
    }
    if (kind == 4) rng->SkipAhead(n, kStreams[st]);
    if (kind == 5) {
      auto* c = new iqs::RandomNumberGenerator<B>(rng);
      delete rng;
      rng = c;
    }
    if (kind <= 3)
      for (int j = 0; j < n; ++j) std::printf("%.17g\n", (double)v[j]);
  }
  std::printf("counts %zu %zu %zu\n", rng->GetNumGeneratedOrSkippedPoolNumbers(),
              rng->GetNumGeneratedOrSkippedStateNumbers(), rng->GetNumGeneratedOrSkippedLocalNumbers());
  delete rng;
}

template <class T>
void read_state(iqs::QubitRegister<T>& r, unsigned n) {
  for (std::size_t i = 0; i < (std::size_t(1) << n); ++i) {
    double re, im;
    std::cin >> re >> im;
    r.SetGlobalAmplitude(i, T(re, im));
  }
}

template <class T>
void print_state(iqs::QubitRegister<T>& r) {
  for (std::size_t i = 0; i < r.GlobalSize(); ++i) {
    const T v = r.GetGlobalAmplitude(i);
    std::printf("%.17g %.17g\n", (double)v.real(), (double)v.imag());
  }
}

template <class T>
void run_noise(unsigned n, std::size_t seed, double T1, double T2, int steps) {
  using B = typename iqs::QubitRegister<T>::BaseType;
  iqs::QubitRegister<T> r(n, "base", 0);
  read_state(r, n);
  iqs::RandomNumberGenerator<B> rng;
  rng.SetSeedStreamPtrs(seed);
  r.SetRngPtr(&rng);
  r.SetNoiseTimescales((B)T1, (B)T2);
  for (int i = 0; i < steps; ++i) {
    unsigned q;
    double d;
    std::cin >> q >> d;
    r.ApplyNoiseGate(q, (B)d);
  }
  print_state(r);
  std::printf("counts %zu %zu %zu\n", rng.GetNumGeneratedOrSkippedPoolNumbers(),
              rng.GetNumGeneratedOrSkippedStateNumbers(), rng.GetNumGeneratedOrSkippedLocalNumbers());
}

template <class T>
void run_noisy(unsigned n, unsigned seed, double T1, double T2, double Ts, double Td, int nprog) {
  using B = typename iqs::QubitRegister<T>::BaseType;
  iqs::NoisyQureg<T> r(n, seed, (B)T1, (B)T2);
  r.Initialize("base", 0);
  r.SetGateDurations((B)Ts, (B)Td);
  for (int i = 0; i < nprog; ++i) {
    int kind;
    unsigned a, b;
    double ang, m[8];
    std::cin >> kind >> a >> b >> ang;
    for (double& x : m) std::cin >> x;
    TM2x2<T> u;
    for (int k = 0; k < 4; ++k) u(k / 2, k % 2) = T((B)m[2 * k], (B)m[2 * k + 1]);
    if (kind == 0) r.ApplyHadamard(a);
    if (kind == 1) r.ApplyRotationX(a, (B)ang);
    if (kind == 2) r.ApplyRotationY(a, (B)ang);
    if (kind == 3) r.ApplyRotationZ(a, (B)ang);
    if (kind == 4) r.ApplyCPauliX(a, b);
    if (kind == 5) r.ApplyControlled1QubitGate(a, b, u);
    if (kind == 6) r.Apply1QubitGate(a, u);
    if (kind == 7) r.ApplyNoiseGatesOnAllQubits();
  }
  print_state(r);
  std::printf("counts %u %u", r.GetOneQubitExperimentalGateCount(), r.GetTwoQubitExperimentalGateCount());
  for (unsigned x = 0; x < n; ++x)
    for (unsigned y = 0; y < n; ++y) std::printf(" %u", r.GetExperimentalGateCount(x, y));
  std::printf("\n");
}

template <class T, unsigned M>
void run_channel(unsigned n, std::size_t seed, int steps) {
  using B = typename iqs::QubitRegister<T>::BaseType;
  std::vector<T> ev(M);
  std::vector<std::vector<T>> vecs(M, std::vector<T>(M));
  for (auto& e : ev) {
    double re, im;
    std::cin >> re >> im;
    e = T(re, im);
  }
  for (auto& row : vecs)
    for (auto& e : row) {
      double re, im;
      std::cin >> re >> im;
      e = T(re, im);
    }
  iqs::ChiMatrix<T, M, 32> chi;
  chi.SetEigenSystem(ev, vecs);
  iqs::QubitRegister<T> r(n, "base", 0);
  read_state(r, n);
  iqs::RandomNumberGenerator<B> rng;
  rng.SetSeedStreamPtrs(seed);
  r.SetRngPtr(&rng);
  for (int i = 0; i < steps; ++i) {
    if constexpr (M == 4) {
      unsigned q;
      std::cin >> q;
      r.ApplyChannel(q, chi);
    } else {
      unsigned q1, q2;
      std::cin >> q1 >> q2;
      r.ApplyChannel(q1, q2, chi);
    }
  }
  print_state(r);
  std::printf("sign %.17g\n", (double)r.GetOverallSignOfChannels());
}

template <class T>
void channel_dispatch(unsigned n, std::size_t seed, unsigned M, int steps) {
  if (M == 4) run_channel<T, 4>(n, seed, steps);
  else run_channel<T, 16>(n, seed, steps);
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 2) {
    std::fprintf(stderr, "usage: noise_driver rng|eigen|noise|noisy|channel < case\n");
    return 2;
  }
  const std::string mode = argv[1];
  try {
    if (mode == "eigen") {
      iqs::ChiMatrix<ComplexDP, 2> chi = {{1., 3.}, {3., 7.}};
      chi.SolveEigenSystem();
      for (unsigned k = 0; k < 2; ++k) {
        const auto v = chi.GetEigenVector(k);
        std::printf("%.17g %.17g %.17g %.17g %.17g\n", chi.GetEigenValue(k).real(), v[0].real(), v[0].imag(),
                    v[1].real(), v[1].imag());
      }
      return 0;
    }
    int prec;
    std::cin >> prec;
    if (mode == "rng") {
      std::size_t seed;
      int nops;
      std::cin >> seed >> nops;
      if (prec) run_rng<float>(seed, nops);
      else run_rng<double>(seed, nops);
    } else if (mode == "noise") {
      unsigned n;
      std::size_t seed;
      double T1, T2;
      int steps;
      std::cin >> n >> seed >> T1 >> T2 >> steps;
      if (prec) run_noise<ComplexSP>(n, seed, T1, T2, steps);
      else run_noise<ComplexDP>(n, seed, T1, T2, steps);
    } else if (mode == "noisy") {
      unsigned n, seed;
      double T1, T2, Ts, Td;
      int nprog;
      std::cin >> n >> seed >> T1 >> T2 >> Ts >> Td >> nprog;
      if (prec) run_noisy<ComplexSP>(n, seed, T1, T2, Ts, Td, nprog);
      else run_noisy<ComplexDP>(n, seed, T1, T2, Ts, Td, nprog);
    } else if (mode == "channel") {
      unsigned n, M;
      std::size_t seed;
      int steps;
      std::cin >> n >> seed >> M >> steps;
      if (prec) channel_dispatch<ComplexSP>(n, seed, M, steps);
      else channel_dispatch<ComplexDP>(n, seed, M, steps);
    } else {
      std::fprintf(stderr, "unknown mode %s\n", mode.c_str());
      return 2;
    }
  } catch (const std::exception& e) {
    std::fprintf(stderr, "error: %s\n", e.what());
    return 1;
  }
  return 0;
}
