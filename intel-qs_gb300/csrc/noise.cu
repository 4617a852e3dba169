// Host side of the stochastic-noise paths: the reference's random number streams, the
// Pauli-twirl noise gate, and chi-matrix channels turned into one 1- or 2-qubit gate per draw.
// The gate itself runs through the ordinary gate kernels.
//
// Random numbers (include/rng_utils.hpp, src/rng_utils.cpp:13-225 of intel/intel-qs): three
// std::mt19937 streams -- "pool" (seed), "state" (seed + 1 + state id) and "local" (seed + 1 +
// number of states + pool rank) -- sharing one std::uniform_real_distribution and one
// std::normal_distribution per base type, with per-stream counts. A uniform draw counts 1,
// a Gaussian draw 2, a skip draws and discards uniforms. Values equal the reference's because the
// same standard-library generator and distributions produce them; that is why this stays C++.
//
// Arithmetic of the noise gate and of the channel gates follows the reference's expressions
// term for term in the base type (float for ComplexSP, double for ComplexDP), so that single
// precision rounds the same way.
#include <algorithm>
#include <cmath>
#include <complex>
#include <random>
#include <vector>

#include "iqsg_internal.cuh"

struct iqsg_rng {
  uint64_t seed = 0;
  uint64_t stream_seed[3] = {0, 1, 2};  // seeds of the pool, state and local streams
  uint64_t count[3] = {0, 0, 0};
  std::mt19937 gen[3];
  std::uniform_real_distribution<double> ud{0.0, 1.0};
  std::normal_distribution<double> nd{0.0, 1.0};
  std::uniform_real_distribution<float> uf{0.0f, 1.0f};
  std::normal_distribution<float> nf{0.0f, 1.0f};

  // Pool stream: seed; state stream: seed + 1 + state id; local stream: seed + 1 + number of
  // states + pool rank (src/rng_utils.cpp:84-99).
  void set_seed(uint64_t s, uint64_t num_states = 1, uint64_t state_id = 0, uint64_t pool_rank = 0) {
    seed = s;
    stream_seed[0] = s;
    stream_seed[1] = s + 1 + state_id;
    stream_seed[2] = s + 1 + num_states + pool_rank;
    for (int st = 0; st < 3; ++st) {
      count[st] = 0;
      gen[st].seed((std::mt19937::result_type)stream_seed[st]);
    }
  }
  // Uniform numbers in [a, b) as a + (b - a) * u, u in [0, 1) (src/rng_utils.cpp:130-163).
  template <typename B>
  void uniform(B* out, uint64_t n, B a, B b, int st) {
    count[st] += n;
    for (uint64_t i = 0; i < n; ++i) {
      const B u = std::is_same<B, double>::value ? (B)ud(gen[st]) : (B)uf(gen[st]);
      if (out) out[i] = a + (b - a) * u;
    }
  }
  template <typename B>
  void gaussian(B* out, uint64_t n, int st) {
    count[st] += 2 * n;  // the reference counts two uniform numbers per Gaussian
    for (uint64_t i = 0; i < n; ++i) out[i] = std::is_same<B, double>::value ? (B)nd(gen[st]) : (B)nf(gen[st]);
  }
};

// The Gaussian source of NoisyQureg (include/NoisyQureg.hpp:47-66): std::default_random_engine
// seeded once, one std::normal_distribution of the base type.
struct iqsg_noise_engine {
  std::default_random_engine gen;
  std::normal_distribution<double> nd{0.0, 1.0};
  std::normal_distribution<float> nf{0.0f, 1.0f};
};

using namespace iqsg;

namespace {

int check_prec(int precision, const char* what) {
  if (precision != IQSG_COMPLEX_DP && precision != IQSG_COMPLEX_SP)
    return fail(IQSG_EINVAL, "%s: unknown precision %d", what, precision);
  return IQSG_OK;
}

int check_stream(int stream, const char* what) {
  if (stream < 0 || stream > 2) return fail(IQSG_EINVAL, "%s: stream %d (0 pool, 1 state, 2 local)", what, stream);
  return IQSG_OK;
}

template <typename B>
void skip(iqsg_rng* r, uint64_t n, int stream) {
  r->uniform<B>(nullptr, n, B(0), B(1), stream);
}

// Noise gate of src/qureg_noisysimul.cpp:33-85 (and NoisyQureg::NoiseGate,
// include/NoisyQureg.hpp:252-310) from three standard Gaussian draws g.
template <typename B>
int noise_gate(B T1, B T2, B duration, const double* g, double* m8) {
  using C = std::complex<B>;
  B p_X, p_Y, p_Z;
  p_X = (1. - std::exp(-duration / T1)) / 4.;
  p_Y = (1. - std::exp(-duration / T1)) / 4.;
  p_Z = (1. - std::exp(-duration / T2)) / 2. + (1. - std::exp(-duration / T1)) / 4.;
  if (!(p_X > 0 && p_Y > 0 && p_Z > 0))
    return fail(IQSG_EINVAL, "noise gate: probabilities %g %g %g are not positive (check T1, T2 and duration)",
                (double)p_X, (double)p_Y, (double)p_Z);
  B s_X, s_Y, s_Z;
  s_X = std::sqrt(-std::log(1. - p_X));
  s_Y = std::sqrt(-std::log(1. - p_Y));
  s_Z = std::sqrt(-std::log(1. - p_Z));
  B v_X = (B)g[0], v_Y = (B)g[1], v_Z = (B)g[2];
  v_X *= s_X / 2.;
  v_Y *= s_Y / 2.;
  v_Z *= s_Z / 2.;
  // exp(-i vX X) exp(-i vY Y) exp(-i vZ Z) = | A B   -A* C* |
  //                                          | A C    A* B* |
  C A, Bm, Cm;
  A = {std::cos(v_Z), -std::sin(v_Z)};
  Bm = {std::cos(v_X) * std::cos(v_Y), -std::sin(v_X) * std::sin(v_Y)};
  Cm = {std::cos(v_X) * std::sin(v_Y), -std::sin(v_X) * std::cos(v_Y)};
  const C u[4] = {A * Bm, -std::conj(A) * std::conj(Cm), A * Cm, std::conj(A) * std::conj(Bm)};
  for (int i = 0; i < 4; ++i) {
    m8[2 * i] = (double)u[i].real();
    m8[2 * i + 1] = (double)u[i].imag();
  }
  return IQSG_OK;
}

// ---- chi matrices ----

using cplx = std::complex<double>;

// Eigen-decomposition of a Hermitian M x M matrix by cyclic complex Jacobi rotations. Each
// rotation first turns a[p][q] real with a diagonal phase, then zeroes it with a real plane
// rotation (tan 2t = 2|a_pq| / (a_qq - a_pp)). Returns eigenvalues (real) and unit eigenvectors
// (column k of v).
void hermitian_jacobi(std::vector<cplx>& a, unsigned M, std::vector<double>& w, std::vector<cplx>& v) {
  v.assign((size_t)M * M, cplx(0, 0));
  for (unsigned i = 0; i < M; ++i) v[i * M + i] = 1;
  auto at = [&](unsigned i, unsigned j) -> cplx& { return a[(size_t)i * M + j]; };
  double fro = 0;
  for (auto& x : a) fro += std::norm(x);
  const double tol = 1e-32 * std::max(fro, 1e-300);
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0;
    for (unsigned p = 0; p < M; ++p)
      for (unsigned q = p + 1; q < M; ++q) off += std::norm(at(p, q));
    if (off <= tol) break;
    for (unsigned p = 0; p < M; ++p)
      for (unsigned q = p + 1; q < M; ++q) {
        const double mag = std::abs(at(p, q));
        if (mag == 0) continue;
        const cplx ph = at(p, q) / mag;  // e^{i phi}
        const double app = at(p, p).real(), aqq = at(q, q).real();
        const double t = 0.5 * std::atan2(2 * mag, aqq - app);
        const double c = std::cos(t), s = std::sin(t);
        // U on (p, q): [[c, s], [-s e^{-i phi}, c e^{-i phi}]]
        const cplx u00 = c, u01 = s, u10 = -s * std::conj(ph), u11 = c * std::conj(ph);
        for (unsigned k = 0; k < M; ++k) {  // a <- a U (columns p, q)
          const cplx akp = at(k, p), akq = at(k, q);
          at(k, p) = akp * u00 + akq * u10;
          at(k, q) = akp * u01 + akq * u11;
        }
        for (unsigned k = 0; k < M; ++k) {  // a <- U^H a (rows p, q)
          const cplx apk = at(p, k), aqk = at(q, k);
          at(p, k) = std::conj(u00) * apk + std::conj(u10) * aqk;
          at(q, k) = std::conj(u01) * apk + std::conj(u11) * aqk;
        }
        at(p, q) = at(q, p) = 0;
        at(p, p) = at(p, p).real();
        at(q, q) = at(q, q).real();
        for (unsigned k = 0; k < M; ++k) {  // v <- v U
          const cplx vkp = v[(size_t)k * M + p], vkq = v[(size_t)k * M + q];
          v[(size_t)k * M + p] = vkp * u00 + vkq * u10;
          v[(size_t)k * M + q] = vkp * u01 + vkq * u11;
        }
      }
  }
  w.resize(M);
  for (unsigned i = 0; i < M; ++i) w[i] = at(i, i).real();
}

// The reference's NormalizeEigenProbAndRenormalizeEigenVect (src/chi_matrix.cpp:166-200) in the
// base type: p_k = |E_k| / sum |E_k|, cumulative sums, eigenvectors scaled by sqrt(sum |E_k|).
template <typename B>
int normalize_eigen(unsigned M, const double* evals, double* evecs, double* probs, double* cumprobs) {
  using C = std::complex<B>;
  B normalization = 0;
  std::vector<B> ep(M), ec(M);
  for (unsigned k = 0; k < M; ++k) {
    const C e((B)evals[2 * k], (B)evals[2 * k + 1]);
    if (!(std::abs(std::imag(e)) < 1.0e-14))
      return fail(IQSG_EINVAL, "chi matrix: eigenvalue %u is not real (imaginary part %g)", k, (double)std::imag(e));
    const B p = std::abs(std::real(e));
    ep[k] = p;
    normalization += p;
    ec[k] = normalization;
  }
  if (normalization != 0 && normalization != 1) {
    for (unsigned k = 0; k < M; ++k) {
      ep[k] /= normalization;
      ec[k] /= normalization;
    }
    const B scale = std::sqrt(normalization);
    for (size_t i = 0; i < (size_t)M * M; ++i) {
      C x((B)evecs[2 * i], (B)evecs[2 * i + 1]);
      x *= scale;
      evecs[2 * i] = (double)x.real();
      evecs[2 * i + 1] = (double)x.imag();
    }
  }
  for (unsigned k = 0; k < M; ++k) {
    probs[k] = (double)ep[k];
    cumprobs[k] = (double)ec[k];
  }
  return IQSG_OK;
}

// One draw of a channel (src/qureg_apply_channel.cpp:17-106): a uniform r on the "state" stream
// selects the first k with r <= cumprob[k]; eigenvector k, read as coefficients on the Pauli
// basis {I, X, Y, Z} (ordered I.I, I.X, ..., Z.Z for two qubits), becomes the gate. The element
// expressions (including the lower triangle of the 4x4 taken as the conjugate of the upper one)
// are the reference's, kept term for term so both precisions round identically.
template <typename B>
int channel_gate(iqsg_rng* r, unsigned M, const double* cumprobs, const double* evecs, double* gate, unsigned* k_out) {
  using C = std::complex<B>;
  B rv;
  r->uniform<B>(&rv, 1, B(0), B(1), 1);
  unsigned k = 0;
  while (rv > (B)cumprobs[k]) {
    ++k;
    if (k >= M) return fail(IQSG_EINVAL, "channel: cumulative probabilities do not reach 1 (draw %g)", (double)rv);
  }
  *k_out = k;
  std::vector<C> e(M);
  for (unsigned i = 0; i < M; ++i) e[i] = C((B)evecs[2 * ((size_t)k * M + i)], (B)evecs[2 * ((size_t)k * M + i) + 1]);
  const C I(0., 1.);
  auto put = [&](unsigned dim, unsigned row, unsigned col, C x) {
    gate[2 * (row * dim + col)] = (double)x.real();
    gate[2 * (row * dim + col) + 1] = (double)x.imag();
  };
  if (M == 4) {
    put(2, 0, 0, e[0] + e[3]);
    put(2, 0, 1, e[1] - I * e[2]);
    put(2, 1, 0, e[1] + I * e[2]);
    put(2, 1, 1, e[0] - e[3]);
    return IQSG_OK;
  }
  C m[4][4];
  m[0][0] = e[0] + e[3] + e[12] + e[15];
  m[1][1] = e[0] - e[3] + e[12] - e[15];
  m[2][2] = e[0] + e[3] - e[12] - e[15];
  m[3][3] = e[0] - e[3] - e[12] + e[15];
  m[0][1] = e[1] + e[13] - I * (e[2] + e[14]);
  m[1][0] = std::conj(m[0][1]);
  m[2][3] = e[1] - e[13] - I * (e[2] - e[14]);
  m[3][2] = std::conj(m[2][3]);
  m[0][2] = e[4] + e[7] - I * (e[8] + e[11]);
  m[1][3] = e[4] - e[7] - I * (e[8] - e[11]);
  m[0][3] = e[5] - e[10] - I * (e[9] + e[6]);
  m[1][2] = e[5] + e[10] - I * (e[9] - e[6]);
  m[2][0] = std::conj(m[0][2]);
  m[3][1] = std::conj(m[1][3]);
  m[3][0] = std::conj(m[0][3]);
  m[2][1] = std::conj(m[1][2]);
  for (unsigned i = 0; i < 4; ++i)
    for (unsigned j = 0; j < 4; ++j) put(4, i, j, m[i][j]);
  return IQSG_OK;
}

}  // namespace

// ---- random number streams ----

extern "C" int iqsg_rng_create(iqsg_rng** out) {
  if (!out) return fail(IQSG_EINVAL, "iqsg_rng_create: null output");
  *out = new iqsg_rng();
  return IQSG_OK;
}

extern "C" void iqsg_rng_destroy(iqsg_rng* r) { delete r; }

extern "C" int iqsg_rng_clone(const iqsg_rng* src, int precision, iqsg_rng** out) {
  if (!src || !out) return fail(IQSG_EINVAL, "iqsg_rng_clone: null argument");
  int st = check_prec(precision, "iqsg_rng_clone");
  if (st) return st;
  auto* r = new iqsg_rng();
  r->set_seed(src->seed);
  for (int s = 0; s < 3; ++s) {
    r->stream_seed[s] = src->stream_seed[s];
    r->gen[s].seed((std::mt19937::result_type)r->stream_seed[s]);
  }
  for (int s = 0; s < 3; ++s) {
    if (precision == IQSG_COMPLEX_DP)
      skip<double>(r, src->count[s], s);
    else
      skip<float>(r, src->count[s], s);
  }
  *out = r;
  return IQSG_OK;
}

extern "C" int iqsg_rng_set_seed(iqsg_rng* r, uint64_t seed) {
  if (!r) return fail(IQSG_EINVAL, "null random number generator");
  r->set_seed(seed);
  return IQSG_OK;
}

extern "C" int iqsg_rng_set_seed_pool(iqsg_rng* r, uint64_t seed, unsigned num_states, unsigned state_id,
                                      unsigned pool_rank) {
  if (!r) return fail(IQSG_EINVAL, "null random number generator");
  if (num_states == 0 || state_id >= num_states)
    return fail(IQSG_EINVAL, "iqsg_rng_set_seed_pool: state %u of %u states", state_id, num_states);
  r->set_seed(seed, num_states, state_id, pool_rank);
  return IQSG_OK;
}

extern "C" int iqsg_rng_skip(iqsg_rng* r, int precision, uint64_t n, int stream) {
  if (!r) return fail(IQSG_EINVAL, "null random number generator");
  int st = check_prec(precision, "iqsg_rng_skip");
  if (!st) st = check_stream(stream, "iqsg_rng_skip");
  if (st) return st;
  if (precision == IQSG_COMPLEX_DP)
    skip<double>(r, n, stream);
  else
    skip<float>(r, n, stream);
  return IQSG_OK;
}

extern "C" int iqsg_rng_uniform(iqsg_rng* r, int precision, double* out, uint64_t n, double a, double b, int stream) {
  if (!r || (n && !out)) return fail(IQSG_EINVAL, "iqsg_rng_uniform: null argument");
  int st = check_prec(precision, "iqsg_rng_uniform");
  if (!st) st = check_stream(stream, "iqsg_rng_uniform");
  if (st) return st;
  if (precision == IQSG_COMPLEX_DP) {
    r->uniform<double>(out, n, a, b, stream);
  } else {
    std::vector<float> f(n);
    r->uniform<float>(f.data(), n, (float)a, (float)b, stream);
    for (uint64_t i = 0; i < n; ++i) out[i] = f[i];
  }
  return IQSG_OK;
}

extern "C" int iqsg_rng_gaussian(iqsg_rng* r, int precision, double* out, uint64_t n, int stream) {
  if (!r || (n && !out)) return fail(IQSG_EINVAL, "iqsg_rng_gaussian: null argument");
  int st = check_prec(precision, "iqsg_rng_gaussian");
  if (!st) st = check_stream(stream, "iqsg_rng_gaussian");
  if (st) return st;
  if (precision == IQSG_COMPLEX_DP) {
    r->gaussian<double>(out, n, stream);
  } else {
    std::vector<float> f(n);
    r->gaussian<float>(f.data(), n, stream);
    for (uint64_t i = 0; i < n; ++i) out[i] = f[i];
  }
  return IQSG_OK;
}

// RandomIntegersInRange (src/rng_utils.cpp:168-190): floor(a + u (b - a)) in the base type.
extern "C" int iqsg_rng_integers(iqsg_rng* r, int precision, int* out, uint64_t n, int a, int b, int stream) {
  if (!r || (n && !out)) return fail(IQSG_EINVAL, "iqsg_rng_integers: null argument");
  int st = check_prec(precision, "iqsg_rng_integers");
  if (!st) st = check_stream(stream, "iqsg_rng_integers");
  if (st) return st;
  auto draw = [&](auto zero) {
    using B = decltype(zero);
    for (uint64_t i = 0; i < n; ++i) {
      B u;
      r->uniform<B>(&u, 1, B(0), B(1), stream);
      u = (B)a + u * B(b - a);
      out[i] = (int)std::floor(u);
    }
  };
  if (precision == IQSG_COMPLEX_DP)
    draw(0.0);
  else
    draw(0.0f);
  return IQSG_OK;
}

extern "C" int iqsg_rng_info(const iqsg_rng* r, uint64_t* seed, uint64_t* counts) {
  if (!r) return fail(IQSG_EINVAL, "null random number generator");
  if (seed) *seed = r->seed;
  if (counts)
    for (int s = 0; s < 3; ++s) counts[s] = r->count[s];
  return IQSG_OK;
}

// Initialize("rand") (src/qureg_init.cpp:256-333) without the final normalisation: a copy of the
// generator (same seed, the stream's count skipped) fills the amplitudes with uniforms in [-1, 1),
// then the generator itself skips the 2 * 2^n numbers.
extern "C" int iqsg_init_random(iqsg_state* h, iqsg_rng* r, int stream) {
  if (!h || !r) return fail(IQSG_EINVAL, "iqsg_init_random: null argument");
  int st = check_stream(stream, "iqsg_init_random");
  if (st) return st;
  if (r->seed == 0) return fail(IQSG_EINVAL, "iqsg_init_random: the generator needs a nonzero seed");
  st = iqsg_init_uniform_random(h, r->stream_seed[stream], r->count[stream], -1.0, 1.0);
  if (st) return st;
  if (h->prec == IQSG_COMPLEX_DP)
    skip<double>(r, 2 * h->N, stream);
  else
    skip<float>(r, 2 * h->N, stream);
  return IQSG_OK;
}

// ---- noise gates ----

extern "C" int iqsg_noise_gate_matrix(int precision, double T1, double T2, double duration, const double* gauss,
                                      double* m8) {
  if (!gauss || !m8) return fail(IQSG_EINVAL, "iqsg_noise_gate_matrix: null argument");
  int st = check_prec(precision, "iqsg_noise_gate_matrix");
  if (st) return st;
  if (precision == IQSG_COMPLEX_DP) return noise_gate<double>(T1, T2, duration, gauss, m8);
  return noise_gate<float>((float)T1, (float)T2, (float)duration, gauss, m8);
}

extern "C" int iqsg_noise_gate_draw(iqsg_rng* r, int precision, double T1, double T2, double duration, double* m8) {
  if (!r || !m8) return fail(IQSG_EINVAL, "iqsg_noise_gate_draw: null argument");
  int st = check_prec(precision, "iqsg_noise_gate_draw");
  if (st) return st;
  double g[3];
  // Three separate draws on the "state" stream, shared by the ranks of one state.
  for (int i = 0; i < 3; ++i) {
    st = iqsg_rng_gaussian(r, precision, &g[i], 1, 1);
    if (st) return st;
  }
  return iqsg_noise_gate_matrix(precision, T1, T2, duration, g, m8);
}

extern "C" int iqsg_noise_engine_create(uint32_t seed, iqsg_noise_engine** out) {
  if (!out) return fail(IQSG_EINVAL, "iqsg_noise_engine_create: null output");
  auto* e = new iqsg_noise_engine();
  e->gen.seed(seed);
  *out = e;
  return IQSG_OK;
}

extern "C" void iqsg_noise_engine_destroy(iqsg_noise_engine* e) { delete e; }

extern "C" int iqsg_noise_engine_gaussian(iqsg_noise_engine* e, int precision, double* out, uint64_t n) {
  if (!e || (n && !out)) return fail(IQSG_EINVAL, "iqsg_noise_engine_gaussian: null argument");
  int st = check_prec(precision, "iqsg_noise_engine_gaussian");
  if (st) return st;
  for (uint64_t i = 0; i < n; ++i) out[i] = precision == IQSG_COMPLEX_DP ? e->nd(e->gen) : (double)e->nf(e->gen);
  return IQSG_OK;
}

// ---- chi matrices and channels ----

extern "C" int iqsg_chi_eigensystem(int precision, unsigned M, const double* chi, double* evals, double* evecs,
                                    double* probs, double* cumprobs) {
  if (!chi || !evals || !evecs || !probs || !cumprobs) return fail(IQSG_EINVAL, "iqsg_chi_eigensystem: null argument");
  int st = check_prec(precision, "iqsg_chi_eigensystem");
  if (st) return st;
  if (M == 0 || M > 64) return fail(IQSG_EINVAL, "iqsg_chi_eigensystem: dimension %u (1..64)", M);
  std::vector<cplx> a((size_t)M * M);
  double amax = 0;
  for (size_t i = 0; i < a.size(); ++i) {
    a[i] = cplx(chi[2 * i], chi[2 * i + 1]);
    amax = std::max(amax, std::abs(a[i]));
  }
  for (unsigned i = 0; i < M; ++i)
    for (unsigned j = 0; j <= i; ++j)
      if (std::abs(a[(size_t)i * M + j] - std::conj(a[(size_t)j * M + i])) > 1e-12 * std::max(amax, 1.0))
        return fail(IQSG_EINVAL, "iqsg_chi_eigensystem: chi is not Hermitian at (%u, %u): its eigenvalues are not real",
                    i, j);
  std::vector<double> w;
  std::vector<cplx> v;
  hermitian_jacobi(a, M, w, v);
  // Order: increasing |E_k|, ties by increasing E_k.
  std::vector<unsigned> ord(M);
  for (unsigned k = 0; k < M; ++k) ord[k] = k;
  std::stable_sort(ord.begin(), ord.end(), [&](unsigned x, unsigned y) {
    if (std::abs(w[x]) != std::abs(w[y])) return std::abs(w[x]) < std::abs(w[y]);
    return w[x] < w[y];
  });
  for (unsigned k = 0; k < M; ++k) {
    const unsigned src = ord[k];
    // Phase: the largest component (first one on ties) real and positive.
    unsigned big = 0;
    for (unsigned i = 1; i < M; ++i)
      if (std::abs(v[(size_t)i * M + src]) > std::abs(v[(size_t)big * M + src]) * (1 + 1e-12)) big = i;
    const double mag = std::abs(v[(size_t)big * M + src]);
    const cplx ph = mag > 0 ? std::conj(v[(size_t)big * M + src]) / mag : cplx(1, 0);
    // Standardisation chi = sum_k E_k |E_k><E_k| holds for unit eigenvectors, which these are.
    for (unsigned i = 0; i < M; ++i) {
      const cplx x = v[(size_t)i * M + src] * ph;
      evecs[2 * ((size_t)k * M + i)] = x.real();
      evecs[2 * ((size_t)k * M + i) + 1] = x.imag();
    }
    evals[2 * k] = w[src];
    evals[2 * k + 1] = 0;
  }
  if (precision == IQSG_COMPLEX_SP)
    for (size_t i = 0; i < 2 * (size_t)M * M; ++i) evecs[i] = (double)(float)evecs[i];
  if (precision == IQSG_COMPLEX_SP)
    for (unsigned k = 0; k < 2 * M; ++k) evals[k] = (double)(float)evals[k];
  return precision == IQSG_COMPLEX_DP ? normalize_eigen<double>(M, evals, evecs, probs, cumprobs)
                                      : normalize_eigen<float>(M, evals, evecs, probs, cumprobs);
}

extern "C" int iqsg_chi_normalize(int precision, unsigned M, const double* evals, double* evecs, double* probs,
                                  double* cumprobs) {
  if (!evals || !evecs || !probs || !cumprobs) return fail(IQSG_EINVAL, "iqsg_chi_normalize: null argument");
  int st = check_prec(precision, "iqsg_chi_normalize");
  if (st) return st;
  if (M == 0 || M > 64) return fail(IQSG_EINVAL, "iqsg_chi_normalize: dimension %u (1..64)", M);
  return precision == IQSG_COMPLEX_DP ? normalize_eigen<double>(M, evals, evecs, probs, cumprobs)
                                      : normalize_eigen<float>(M, evals, evecs, probs, cumprobs);
}

extern "C" int iqsg_channel_gate(iqsg_rng* r, int precision, unsigned M, const double* evals, const double* cumprobs,
                                 const double* evecs, double* gate, unsigned* k_out, int* negative) {
  if (!r || !evals || !cumprobs || !evecs || !gate) return fail(IQSG_EINVAL, "iqsg_channel_gate: null argument");
  int st = check_prec(precision, "iqsg_channel_gate");
  if (st) return st;
  if (M != 4 && M != 16) return fail(IQSG_EINVAL, "iqsg_channel_gate: chi dimension %u (4 or 16)", M);
  unsigned k = 0;
  st = precision == IQSG_COMPLEX_DP ? channel_gate<double>(r, M, cumprobs, evecs, gate, &k)
                                    : channel_gate<float>(r, M, cumprobs, evecs, gate, &k);
  if (st) return st;
  if (k_out) *k_out = k;
  if (negative) {
    const double re = precision == IQSG_COMPLEX_DP ? evals[2 * k] : (double)(float)evals[2 * k];
    *negative = re < 0;
  }
  return IQSG_OK;
}
