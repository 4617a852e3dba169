/* iqsg.h -- C ABI of the GB300 state-vector engine (libiqsg.so).
 *
 * This is the drop-in boundary for the gate-application hot path of intel/intel-qs.
 * The reference has no C ABI: its boundary is the C++ class template
 * iqs::QubitRegister<Type> (include/qureg.hpp:127-417). Each entry point below replaces
 * the local (single-rank) branch of one QubitRegister method, cited per function; the
 * C++ header include/iqs_gb300/qureg.hpp and the Python package iqs_gb300 rebuild the
 * QubitRegister API on top of these calls.
 *
 * Conventions
 *  - A register of n qubits holds 2^n complex amplitudes in device memory (HBM),
 *    interleaved (re, im) exactly like std::complex<double> (IQSG_COMPLEX_DP, 16 B)
 *    or std::complex<float> (IQSG_COMPLEX_SP, 8 B), 256-byte aligned.
 *  - Every qubit argument is a data POSITION: bit k of an amplitude's index is
 *    position k. The program-qubit -> position map (iqs::Permutation,
 *    include/permutation.hpp) is kept by the caller, as QubitRegister does.
 *  - Gate matrices are row-major, interleaved, always double precision:
 *    m[2*(r*dim+c)] = Re m_rc, m[2*(r*dim+c)+1] = Im m_rc (TinyMatrix layout,
 *    include/tinymatrix.hpp). An SP register rounds them to float.
 *  - Every call returns an iqsg_status. On failure iqsg_last_error() describes it.
 *    Invalid arguments are rejected before any device work (the reference asserts).
 *  - Work is queued on the register's CUDA stream. Gate calls return without waiting;
 *    calls that return a value (probabilities, norms, amplitudes, ...) wait for it.
 *  - All reductions accumulate in FP64 on the device, in a fixed order (deterministic).
 */
#ifndef IQSG_H
#define IQSG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  IQSG_OK = 0,
  IQSG_EINVAL = 1,   /* invalid argument (qubit position, size, map, null pointer ...) */
  IQSG_ENOMEM = 2,   /* device or pinned-host allocation failed */
  IQSG_EDEVICE = 3,  /* CUDA runtime error (launch failure, no device ...) */
  IQSG_ETIMEOUT = 4, /* a bounded device-side wait gave up */
  IQSG_ENOTSUP = 5   /* valid request this build does not support */
} iqsg_status;

typedef enum { IQSG_COMPLEX_DP = 0, IQSG_COMPLEX_SP = 1 } iqsg_precision;

/* Arithmetic used by ComplexDP gate kernels.
 *  NATIVE: IEEE FP64 fused multiply-adds (the GB300 FP64 pipe: about 0.5 T instr/s).
 *  EMULATED: FP64 storage, products and sums in double-float (two FP32 words, about
 *            48-bit significand) on the FP32 pipe, rounded back to FP64 on store.
 *  ComplexSP registers always compute in FP32. */
typedef enum { IQSG_MATH_NATIVE = 0, IQSG_MATH_EMULATED = 1 } iqsg_math;

typedef struct iqsg_state iqsg_state;

/* ---- errors, version ---------------------------------------------------------------- */

/* Text of the last error raised on the calling thread ("" if none). */
const char* iqsg_last_error(void);
/* Library version as major*10000 + minor*100 + patch. */
int iqsg_version(void);

/* ---- lifecycle ------------------------------------------------------------------------ */

/* Devices: a register lives on the device that is current (cudaSetDevice) when it is created,
 * and every call on it must be made with that device current, as with any CUDA runtime
 * object. Several devices may be used from one process this way. */

/* Allocate a register of num_qubits qubits on the current CUDA device and zero it.
 * stream: a cudaStream_t to queue work on, or NULL for a stream owned by the register.
 * Replaces QubitRegister(n, style, base, tmp) allocation: src/qureg_init.cpp:149-188. */
int iqsg_create(unsigned num_qubits, int precision, void* stream, iqsg_state** out);

/* Wrap caller-owned device memory (2^n amplitudes, 256-B aligned) without copying.
 * destroy() does not free it. Replaces the imported-state constructor
 * QubitRegister(n, Type* state, tmp): src/qureg_init.cpp:193-200. */
int iqsg_create_from_device(unsigned num_qubits, int precision, void* device_amps, void* stream,
                            iqsg_state** out);

/* Deep copy (device to device) into a new register on the same stream.
 * Replaces the copy constructor: src/qureg_init.cpp:364-379. */
int iqsg_clone(const iqsg_state* src, iqsg_state** out);

/* Free the register (and its device memory unless wrapped). Replaces ~QubitRegister:
 * src/qureg_init.cpp:452-461. Accepts NULL. */
int iqsg_destroy(iqsg_state* h);

/* Query size, precision and the device address of amplitude 0. */
int iqsg_info(const iqsg_state* h, unsigned* num_qubits, int* precision, void** device_amps);

/* Select the ComplexDP gate arithmetic (iqsg_math). Default: IQSG_MATH_NATIVE. */
int iqsg_set_math(iqsg_state* h, int math);

/* Wait for all work queued on the register's stream. */
int iqsg_synchronize(iqsg_state* h);

/* ---- initialisation and amplitude access ------------------------------------------------ */

/* Set every amplitude to (re, im). Replaces InitializationWithSameAmplitudeEverywhere:
 * src/qureg_utils.cpp:173-184 (and the "++++" style of Initialize, :342-346). */
int iqsg_fill(iqsg_state* h, double re, double im);

/* Zero the register and set amplitude data_index to 1: Initialize("base", i) with the
 * index already mapped to data order, src/qureg_init.cpp:242-249 and :335-340. */
int iqsg_init_basis(iqsg_state* h, uint64_t data_index);

/* Write / read one amplitude at a data index. Replace SetGlobalAmplitude /
 * GetGlobalAmplitude after program2data_ (src/qureg_utils.cpp:78-121). */
int iqsg_set_amplitude(iqsg_state* h, uint64_t data_index, double re, double im);
int iqsg_get_amplitude(iqsg_state* h, uint64_t data_index, double* re_im);

/* Copy count amplitudes between host memory (in the register's own precision,
 * interleaved) and the register, starting at amplitude offset. Synchronous.
 * The reference exposes its host array directly (RawState(), operator[]:
 * include/qureg.hpp:150-166); this is the explicit host <-> HBM transfer. */
int iqsg_upload(iqsg_state* h, const void* host, uint64_t offset, uint64_t count);
int iqsg_download(iqsg_state* h, void* host, uint64_t offset, uint64_t count);

/* Uniform random amplitudes: the real and imaginary parts, interleaved in data order, are the
 * values a + (b - a) u of std::uniform_real_distribution<T>(0, 1) over std::mt19937(seed), T the
 * register's base type, after discarding the first `skip` values -- the numbers the reference's
 * RandomNumberGenerator stream with that seed gives (src/rng_utils.cpp:84-160), as used by
 * Initialize("rand") (src/qureg_init.cpp:253-330; normalise afterwards). Generated on the host. */
int iqsg_init_uniform_random(iqsg_state* h, uint64_t seed, uint64_t skip, double a, double b);

/* ---- random numbers, noise gates, chi-matrix channels (host side; the gates they produce go
 * through iqsg_apply_1q / iqsg_apply_2q) ---- */

/* Random number streams with the structure of the reference's RandomNumberGenerator
 * (include/rng_utils.hpp:46-130, src/rng_utils.cpp:13-225): three std::mt19937 streams,
 * 0 "pool" (seed), 1 "state" (seed + 1 + state id) and 2 "local" (seed + 1 + number of states +
 * pool rank; see iqsg_rng_set_seed_pool) sharing one std::uniform_real_distribution and one
 * std::normal_distribution per base type, with per-stream counts: a uniform counts 1, a Gaussian
 * 2, a skip draws and discards uniforms. `precision` (IQSG_COMPLEX_SP / _DP) picks the base type
 * (float / double) as the reference's template argument does; values are returned as doubles. */
typedef struct iqsg_rng iqsg_rng;
int iqsg_rng_create(iqsg_rng** out);
void iqsg_rng_destroy(iqsg_rng* r);
/* Copy constructor (src/rng_utils.cpp:13-20): same seed, each stream's count skipped. */
int iqsg_rng_clone(const iqsg_rng* src, int precision, iqsg_rng** out);
int iqsg_rng_set_seed(iqsg_rng* r, uint64_t seed);                          /* SetSeedStreamPtrs */
/* SetSeedStreamPtrs in a pool of num_states states: the state stream is seeded with
 * seed + 1 + state_id and the local one with seed + 1 + num_states + pool_rank
 * (src/rng_utils.cpp:84-99); iqsg_rng_set_seed is the one-state pool (1, 0, 0). */
int iqsg_rng_set_seed_pool(iqsg_rng* r, uint64_t seed, unsigned num_states, unsigned state_id,
                           unsigned pool_rank);
int iqsg_rng_skip(iqsg_rng* r, int precision, uint64_t n, int stream);       /* SkipAhead */
int iqsg_rng_uniform(iqsg_rng* r, int precision, double* out, uint64_t n, double a, double b,
                     int stream);                                            /* UniformRandomNumbers */
int iqsg_rng_gaussian(iqsg_rng* r, int precision, double* out, uint64_t n, int stream);
int iqsg_rng_integers(iqsg_rng* r, int precision, int* out, uint64_t n, int a, int b,
                      int stream);                                           /* RandomIntegersInRange */
int iqsg_rng_info(const iqsg_rng* r, uint64_t* seed, uint64_t* counts /* [3] */);
/* Initialize("rand") (src/qureg_init.cpp:256-333) without its final normalisation: amplitudes
 * uniform in [-1, 1) from a copy of r on the stream (0 pool, 2 local), then r skips 2 * 2^n. */
int iqsg_init_random(iqsg_state* h, iqsg_rng* r, int stream);

/* The Pauli-twirl noise gate of ApplyNoiseGate (src/qureg_noisysimul.cpp:33-85) as a 2x2
 * row-major complex matrix, from three standard Gaussians `gauss`, computed in the base type. */
int iqsg_noise_gate_matrix(int precision, double T1, double T2, double duration, const double* gauss,
                           double* m8);
/* The same with the three Gaussians drawn from r's "state" stream, as ApplyNoiseGate draws them. */
int iqsg_noise_gate_draw(iqsg_rng* r, int precision, double T1, double T2, double duration, double* m8);
/* NoisyQureg's own Gaussian source (include/NoisyQureg.hpp:47-66): std::default_random_engine
 * seeded with `seed` and a std::normal_distribution of the base type. */
typedef struct iqsg_noise_engine iqsg_noise_engine;
int iqsg_noise_engine_create(uint32_t seed, iqsg_noise_engine** out);
void iqsg_noise_engine_destroy(iqsg_noise_engine* e);
int iqsg_noise_engine_gaussian(iqsg_noise_engine* e, int precision, double* out, uint64_t n);

/* Chi matrices (include/chi_matrix.hpp, src/chi_matrix.cpp): M x M complex, row-major
 * interleaved. iqsg_chi_eigensystem replaces SolveEigenSystem: eigenvalues (2M doubles),
 * standardised eigenvectors (row k = eigenvector k, 2M*M doubles), probabilities |E_k|/sum|E| and
 * their running sums; eigenvectors scaled by sqrt(sum |E|). chi must be Hermitian. Order:
 * increasing |E_k|; phase: largest component real and positive. iqsg_chi_normalize is the
 * reference's NormalizeEigenProbAndRenormalizeEigenVect for an eigensystem given by the caller. */
int iqsg_chi_eigensystem(int precision, unsigned M, const double* chi, double* evals, double* evecs,
                         double* probs, double* cumprobs);
int iqsg_chi_normalize(int precision, unsigned M, const double* evals, double* evecs, double* probs,
                       double* cumprobs);
/* One draw of ApplyChannel (src/qureg_apply_channel.cpp:17-106): a uniform on r's "state" stream
 * selects eigenvector k; `gate` receives the 2x2 (M = 4) or 4x4 (M = 16) matrix to apply with
 * iqsg_apply_1q / iqsg_apply_2q; *negative = 1 when E_k < 0 (the register's overall sign flips). */
int iqsg_channel_gate(iqsg_rng* r, int precision, unsigned M, const double* evals, const double* cumprobs,
                      const double* evecs, double* gate, unsigned* k_out, int* negative);

/* The same copies queued on the register's stream without waiting: they run in order with the
 * register's gates, so a caller can overlap one register's transfers with another register's
 * work. The host memory must stay valid, and unread (upload) or untouched (download), until
 * iqsg_synchronize returns; with pinned host memory the call returns at once. */
int iqsg_upload_async(iqsg_state* h, const void* host, uint64_t offset, uint64_t count);
int iqsg_download_async(iqsg_state* h, void* host, uint64_t offset, uint64_t count);

/* Device-to-device copy of all amplitudes (same size and precision). */
int iqsg_copy(iqsg_state* dst, const iqsg_state* src);

/* ---- gates -------------------------------------------------------------------------- */

/* 2x2 gate on position pos: pairs (i, i + 2^pos) with bit pos of i clear,
 * a0' = m00 a0 + m01 a1, a1' = m10 a0 + m11 a1.
 * Replaces Apply1QubitGate_helper -> Loop_DN: src/qureg_apply1qubitgate.cpp:173-230,
 * src/highperfkernels.cpp:287-380. */
int iqsg_apply_1q(iqsg_state* h, unsigned pos, const double* m);

/* 2x2 gate on tpos applied where bit cpos is 1. Replaces
 * ApplyControlled1QubitGate_helper -> Loop_TN: src/qureg_applyctrl1qubitgate.cpp:228-406,
 * src/highperfkernels.cpp:397-486. */
int iqsg_apply_controlled_1q(iqsg_state* h, unsigned cpos, unsigned tpos, const double* m);

/* 2x2 gate on tpos applied where all num_ctrl control positions are 1 (num_ctrl <= 8).
 * With num_ctrl = 2 and m = X this is the Toffoli gate in one pass; the reference
 * composes it from five controlled gates (src/qureg_applytoffoli.cpp:24-47). */
int iqsg_apply_multi_controlled_1q(iqsg_state* h, unsigned num_ctrl, const unsigned* cpos,
                                   unsigned tpos, const double* m);

/* Dense 4x4 gate; row/column index = 2*b(pos_high) + b(pos_low).
 * Replaces Apply2QubitGate: src/qureg_apply2qubitgate.cpp:14-73. */
int iqsg_apply_2q(iqsg_state* h, unsigned pos_high, unsigned pos_low, const double* m);

/* Swap-type gate: 2x2 m on the {|p_lo=1,p_hi=0>, |p_lo=0,p_hi=1>} subspace, with
 * p_lo = min(p1, p2). Replaces ApplySwap_helper: src/qureg_applyswap.cpp:117-234. */
int iqsg_apply_swaplike(iqsg_state* h, unsigned p1, unsigned p2, const double* m);

/* Diagonal two-qubit gate: amp[i] *= d[2*b(p1) + b(p2)], d = 4 complex entries.
 * Replaces ApplyDiag: src/qureg_applydiag.cpp:55-227. */
int iqsg_apply_diag_2q(iqsg_state* h, unsigned p1, unsigned p2, const double* d);

/* amp[i] *= exp(-i gamma Re diag[i]) with diag a register of the same size.
 * Replaces qaoa::ImplementQaoaLayerBasedOnCostFunction: src/qaoa_features.cpp:248-264. */
int iqsg_apply_cost_phase(iqsg_state* h, const iqsg_state* diag, double gamma);

/* Zero the half of the amplitudes where bit pos != value (no renormalisation).
 * Replaces CollapseQubit: src/qureg_measure.cpp:92-126. */
int iqsg_collapse(iqsg_state* h, unsigned pos, int value);

/* amp[i] *= (re, im). Replaces AmplitudeWiseScalarMultiplication: src/qureg_utils.cpp:189-199. */
int iqsg_scale(iqsg_state* h, double re, double im);

/* amp[i] += (re, im) * x[i]. Replaces AmplitudeWiseSum: src/qureg_utils.cpp:207-231. */
int iqsg_axpy(iqsg_state* h, const iqsg_state* x, double re, double im);

/* Reorder amplitudes from position map old_map to new_map (direct maps: program qubit
 * -> position, n entries each): amp'[new.p2d(old.d2p(i))] = amp[i]. Index placement is
 * bit-exact. Replaces PermuteLocalQubits: src/qureg_permute.cpp:57-105. */
int iqsg_permute(iqsg_state* h, const unsigned* old_map, const unsigned* new_map);

/* ---- fused gate streams ------------------------------------------------------------------ */

/* One gate of a stream for iqsg_apply_ops. Positions are data positions; matrices as above. */
typedef enum {
  IQSG_OP_1Q = 0,       /* 2x2 m on t0 */
  IQSG_OP_CTRL = 1,     /* 2x2 m on t0 where all nctrl positions ctrl[] are 1 */
  IQSG_OP_2Q = 2,       /* dense 4x4 m, row/column index 2*b(t0) + b(t1) */
  IQSG_OP_SWAPLIKE = 3, /* 2x2 m on the {|lo=1,hi=0>, |lo=0,hi=1>} pair of positions t0, t1 */
  IQSG_OP_DIAG2 = 4,    /* amp *= m[2*b(t0) + b(t1)] (4 complex entries) */
  IQSG_OP_PHASE = 5,    /* amp *= m[0] where (index & mask) == value */
  IQSG_OP_GRAD1 = 6,    /* iqsg_adjoint_ops only: grads[value] += Im <lam|M|psi>, M = 2x2 m on t0 */
  IQSG_OP_GRAD2 = 7     /* iqsg_adjoint_ops only: grads[value] += Im <lam|M|psi>, M = 4x4 m,
                           row/column index 2*b(t0) + b(t1) */
} iqsg_op_kind;

typedef struct {
  int32_t kind;
  uint32_t t0, t1;
  uint32_t nctrl;
  uint32_t ctrl[4];
  uint64_t mask, value;
  double m[32];
} iqsg_op;

/* Apply count gates in order, packed into fused sweeps: each sweep loads every group of 2^K
 * amplitudes spanned by up to K target positions once, applies all its gates in registers
 * (diagonal gates and controls on any position ride along) and stores the group once.
 * The result equals applying the gates one by one (bit-identical in native FP64/FP32).
 * *sweeps (may be NULL) receives the number of state passes launched.
 * Replaces the reference's cache-blocked replay of buffered gates, ApplyFusedGates:
 * src/qureg_fusion.cpp:55-94. */
int iqsg_apply_ops(iqsg_state* h, const iqsg_op* ops, unsigned count, unsigned* sweeps);

/* Reverse-mode (adjoint) gradients over two registers of equal size and precision: psi (the
 * circuit state after the gates) and lam (the adjoint state, O psi for E = <psi|O|psi>).
 * The ops list the circuit backwards: for each gate G = exp(-i theta A), first (if theta
 * depends on a parameter) an IQSG_OP_GRAD1/GRAD2 op with M = 2 (d theta / d param) A and
 * value = the parameter index, then G^dagger as a gate op. Gate ops act on both registers;
 * a gradient op adds Im <lam|M|psi> over the whole state into grads[value], which is that
 * gate's share of dE/dparam. Everything is packed into fused two-vector sweeps; sums are
 * FP64 in a fixed order. grads (nparams <= 2048 host doubles) is added to, not overwritten.
 * ComplexDP runs in native FP64 arithmetic whatever iqsg_set_math chose. Waits for the
 * result. The reference has no adjoint path: its gradients come from re-running circuits. */
int iqsg_adjoint_ops(iqsg_state* psi, iqsg_state* lam, const iqsg_op* ops, unsigned count, double* grads,
                     unsigned nparams, unsigned* sweeps);

/* Largest number of target positions per sweep (1..4; 0 restores the default: 4 for
 * ComplexSP, 3 for native ComplexDP, 2 for emulated ComplexDP, which is capped at 3).
 * The reference's counterpart is the log2llc block size of TurnOnFusion:
 * src/qureg_fusion.cpp:12-31. */
int iqsg_set_sweep_width(iqsg_state* h, unsigned kmax);

/* Tuning options of a register (iqsg_set_option). */
typedef enum {
  IQSG_OPT_SWEEP_WIDTH = 0,    /* same as iqsg_set_sweep_width */
  IQSG_OPT_SWEEP_PIPELINE = 1, /* 1: fused passes on registers of 16+ qubits stream tiles through
                                  shared memory with bulk async copies; 0 (default): each thread
                                  loads its groups directly */
  IQSG_OPT_TILE_QUBITS = 2,    /* k > 0: run gate streams (iqsg_apply_ops, iqsg_adjoint_ops) as
                                  tile passes: each pass stages tiles spanning k positions (the
                                  lowest 3 or 4 included; at most 14 for ComplexSP, 13 for
                                  ComplexDP, one less for adjoint passes) in shared memory and
                                  applies every gate of a stretch of the stream that acts inside
                                  them, gates on disjoint positions reordered; 0 (default): register
                                  sweeps only. Not used for emulated ComplexDP arithmetic. */
  IQSG_OPT_NATIVE_SHARE = 3,   /* s in 0..16: in emulated-ComplexDP fused sweeps, s/16 of the warps
                                  apply their groups in native FP64 (the FP64 pipe) while the rest
                                  use double-float FP32 arithmetic; 0 (default): all emulated.
                                  Results differ from s = 0 only by rounding. */
  IQSG_OPT_DF_STORAGE = 4      /* 1 (default): an emulated-ComplexDP gate stream of 3+ sweeps whose
                                  gates are all contractive keeps the state as double-float pairs
                                  (four floats per amplitude, same 16 bytes) between its sweeps,
                                  so values are split once and rounded back to FP64 once per call;
                                  the call still ends with FP64 amplitudes. 0: every sweep reads
                                  and writes FP64. Results differ by rounding only. */
} iqsg_option;

/* One fused sweep (one pass over the state) of a planned gate stream. */
typedef struct {
  unsigned k;          /* active positions of the sweep (0..4) */
  unsigned pos[4];     /* those positions, slot order */
  unsigned ops;        /* operations applied in the sweep */
  unsigned one_qubit;  /* of which 2x2 gates (with or without controls) */
  unsigned two_qubit;  /* dense, swap-type or excitation-preserving 4x4 gates */
  unsigned diagonal;   /* phases and merged CZ runs (any positions, no slot needed) */
} iqsg_sweep_info;

/* The sweeps iqsg_apply_ops would run for `ops` on a register of num_qubits positions in the
 * given precision and math (IQSG_MATH_*) with pass width `width` (0: the default) and default
 * options otherwise -- the fusion plan of the reference's ApplyFusedGates
 * (src/qureg_fusion.cpp:12-94), here one pass per sweep. Host only: allocates nothing, needs no
 * GPU. *nsweeps gets the count; out (cap entries, may be null) one iqsg_sweep_info per sweep;
 * *pair_storage whether the call would keep double-float pairs between the sweeps. */
int iqsg_plan_ops(unsigned num_qubits, int precision, int math, unsigned width, const iqsg_op* ops,
                  unsigned count, iqsg_sweep_info* out, unsigned cap, unsigned* nsweeps, int* pair_storage);

/* Counters of a register: [0] double-float storage runs started by iqsg_apply_ops,
 * [1] kernels those runs launched (one range check and two kernels per sweep, one of which
 * returns at once). */
int iqsg_counters(const iqsg_state* h, uint64_t* counters /* [2] */);

/* Set a tuning option. Results depend on it at most by rounding (tile passes reorder gates on
 * disjoint positions; the native share changes which arithmetic a group gets). */
int iqsg_set_option(iqsg_state* h, int option, int value);

/* ---- reductions (FP64 accumulation; each waits for its result) ------------------------ */

/* Sum of |amp|^2 over indices with bit pos = 1. Replaces GetProbability:
 * src/qureg_measure.cpp:135-178. */
int iqsg_probability(iqsg_state* h, unsigned pos, double* p);

/* <psi|P|psi> for the Pauli string P = prod_k obs[k] on position pos[k]
 * (obs: 1 = X, 2 = Y, 3 = Z; positions distinct), in one read-only pass, plus
 * sum |amp|^2 in *norm2 (may be NULL). Replaces the basis-change + parity reduction of
 * ExpectationValue: src/qureg_expectval.cpp:102-213 (the state is not modified). */
int iqsg_expectation_pauli(iqsg_state* h, unsigned k, const unsigned* pos, const unsigned* obs,
                           double* value, double* norm2);

/* State statistics in one read-only pass, as GoogleStats returns them: stats[0] = entropy
 * -sum p log2 p, stats[1] = -sum log2 p over p > 0 divided by 2^n, stats[2 + i] =
 * sum p^k * (2^n)^(k-1) / k! for k = 2..10 (p = |amp|^2; FP64 sums in a fixed order).
 * stats[0] is Entropy(). Replaces Entropy and GoogleStats: src/qureg_utils.cpp:303-450. */
int iqsg_state_stats(iqsg_state* h, double* stats);

/* sum |amp|^2. ComputeNorm returns its square root: src/qureg_utils.cpp:236-256. */
int iqsg_norm2(iqsg_state* h, double* out);

/* <psi|h> = sum conj(psi_i) h_i, as re_im[2]. Replaces ComputeOverlap:
 * src/qureg_utils.cpp:267-300. */
int iqsg_overlap(iqsg_state* h, const iqsg_state* psi, double* re_im);

/* max_i |h_i - (re, im) x_i|. Replaces MaxAbsDiff: src/qureg_utils.cpp:40-68. */
int iqsg_max_abs_diff(iqsg_state* h, const iqsg_state* x, double re, double im, double* out);

/* sum_i |h_i - x_i|^2. Replaces MaxL2NormDiff: src/qureg_utils.cpp:129-157. */
int iqsg_l2_diff(iqsg_state* h, const iqsg_state* x, double* out);

/* sum_i (Re diag_i)^power |psi_i|^2 for power 1 or 2. Replaces
 * GetExpectationValueFromCostFunction / ...SquaredFromCostFunction:
 * src/qaoa_features.cpp:273-331. */
int iqsg_cost_expectation(iqsg_state* psi, const iqsg_state* diag, int power, double* out);

/* Fill diag with the MaxCut value of every basis state: diag[i] = (cut(d2p(i)), 0) for the
 * graph adj (n*n ints, symmetric, zero diagonal), map = direct position map (may be NULL
 * for identity). *max_cut receives the largest cut. Replaces
 * InitializeVectorAsMaxCutCostFunction: src/qaoa_features.cpp:73-143. */
int iqsg_maxcut_cost(iqsg_state* diag, const int* adj, const unsigned* map, int* max_cut);

/* Weighted MaxCut cost vector: Re diag[x] = sum over edges (u, v) of adj[u*n + v] where the
 * program bits u and v of x differ (adj: n*n doubles, symmetric, zero diagonal), computed in
 * FP64 and stored in the register's precision; *max_cut (may be NULL) receives the largest
 * value. Replaces InitializeVectorAsWeightedMaxCutCostFunction: src/qaoa_features.cpp:153-239. */
int iqsg_weighted_maxcut_cost(iqsg_state* diag, const double* adj, const unsigned* map, double* max_cut);

/* Histogram of |psi_x|^2 over the cost values Re diag[x], FP64 sums in a fixed order:
 *   IQSG_HIST_INTEGER: bin (int)cost, num_bins = max_value + 1
 *                      (GetHistogramFromCostFunction, src/qaoa_features.cpp:335-400);
 *   IQSG_HIST_ROUNDED: bin floor(cost + 1e-7), num_bins = floor(max_value) + 1
 *                      (...WithWeightsRounded, :402-469);
 *   IQSG_HIST_BINNED:  bin floor(cost / bin_width + 1e-7), num_bins = ceil(max_value / bin_width) + 1
 *                      (...WithWeightsBinned, :471-538).
 * num_bins must equal that count (at most 4096). A cost outside [0, max_value] (or, for the
 * weighted modes, outside [-1e-7, max_value + 1e-7]) fails with IQSG_EINVAL, where the
 * reference asserts. Waits for the result. */
typedef enum { IQSG_HIST_INTEGER = 0, IQSG_HIST_ROUNDED = 1, IQSG_HIST_BINNED = 2 } iqsg_hist_mode;
int iqsg_cost_histogram(iqsg_state* psi, const iqsg_state* diag, int mode, double max_value, double bin_width,
                        double* hist, unsigned num_bins);

/* ---- QAOA MaxCut circuits and adjoint gradients ---------------------------------------- */

/* One QAOA layer: amp *= exp(-i gamma H_C) with H_C = 1/2 sum_e w_e Z_u Z_v, then
 * exp(-i beta X_q) (= RX(2 beta)) on every qubit. edges: 2*num_edges data positions
 * (u0, v0, u1, v1, ...); weights: num_edges ints in [0, 255] or NULL for unit weights.
 * The cost phase equals qaoa::ImplementQaoaLayerBasedOnCostFunction with the MaxCut cost
 * vector (src/qaoa_features.cpp:248-264) up to a global phase; the mixer equals
 * ApplyRotationX(q, 2 beta) on every qubit (src/qureg_apply1qubitgate.cpp:277-283). */
int iqsg_qaoa_layer(iqsg_state* h, unsigned num_edges, const unsigned* edges, const int* weights, double gamma,
                    double beta);

/* energy = <psi|O|psi> with O = sum_e w_e Z_u Z_v (= sum of ExpectationValueZZ over edges,
 * src/qureg_expectval.cpp:365-375), *norm2 = <psi|psi> (may be NULL). With lam != NULL also
 * writes lam = O psi, the starting adjoint state of a gradient. */
int iqsg_qaoa_observable(iqsg_state* psi, iqsg_state* lam, unsigned num_edges, const unsigned* edges,
                         const int* weights, double* energy, double* norm2);

/* Adjoint step back through one layer: with psi and lam taken after the layer, returns
 * dE/dgamma and dE/dbeta of that layer and leaves psi, lam undone to before it.
 * No counterpart in the reference (it has no gradients). */
int iqsg_qaoa_layer_backward(iqsg_state* psi, iqsg_state* lam, unsigned num_edges, const unsigned* edges,
                             const int* weights, double gamma, double beta, double* grad_gamma, double* grad_beta);

/* Checkpointed layer: as iqsg_qaoa_layer, and after_cost / after_mixer (registers of the same
 * size) receive the state after the cost phase and after the whole layer. */
int iqsg_qaoa_layer_ckpt(iqsg_state* h, iqsg_state* after_cost, iqsg_state* after_mixer, unsigned num_edges,
                         const unsigned* edges, const int* weights, double gamma, double beta);

/* Adjoint step from checkpoints: only lam is walked back through the layer; the two
 * checkpoints of that layer are read. Returns the layer's dE/dgamma and dE/dbeta.
 * No counterpart in the reference. */
int iqsg_qaoa_layer_backward_ckpt(iqsg_state* lam, const iqsg_state* after_cost, const iqsg_state* after_mixer,
                                  unsigned num_edges, const unsigned* edges, const int* weights, double gamma,
                                  double beta, double* grad_gamma, double* grad_beta);

/* ---- batches of small circuits --------------------------------------------------------- */

/* One Pauli string of an observable, in data positions: xmask = positions with X or Y,
 * zmask = positions with Y or Z, ny = number of Y factors mod 4; P|y> = i^ny (-1)^|y & zmask|
 * |y ^ xmask>. */
typedef struct {
  uint64_t xmask, zmask;
  int32_t ny;
  int32_t pad;
  double coeff;
} iqsg_pauli_term;

typedef struct iqsg_batch iqsg_batch;

/* A batch of count hardware-efficient ansatz instances: instance i has num_qubits[i] (<= 24)
 * qubits and num_layers[i] layers, each layer RZ(phi) then RY(theta) on every qubit and CZ(q,
 * q+1) for q = 0..n-2, starting from |0..0>; its observable is terms_per_instance[i] Pauli
 * strings, taken in order from terms. Parameters per instance: [layer][qubit][phi, theta].
 * Allocates two state vectors per instance. No counterpart in the reference. */
int iqsg_batch_create(unsigned count, const unsigned* num_qubits, const unsigned* num_layers,
                      const unsigned* terms_per_instance, const iqsg_pauli_term* terms, int precision,
                      void* stream, iqsg_batch** out);
int iqsg_batch_destroy(iqsg_batch* b);

/* Evaluate every instance in one persistent launch (CTAs pull instances, largest first, from
 * a work counter), recorded once into a CUDA graph and replayed on later calls: energies[i],
 * and with with_grad the adjoint-mode gradient of every parameter (same layout as params).
 * params, energies and grads are host arrays. */
int iqsg_batch_run(iqsg_batch* b, const double* params, int with_grad, double* energies, double* grads);

/* Launch shape of the persistent kernel (threads per CTA: 32..512, a multiple of 32; CTAs per
 * SM: 1..16); chosen by the autotuner. Invalidates the recorded graphs. */
int iqsg_batch_set_launch(iqsg_batch* b, unsigned threads, unsigned ctas_per_sm);
int iqsg_batch_info(const iqsg_batch* b, uint64_t* num_params, uint64_t* total_amplitudes);

/* ---- allocation-free measurement -------------------------------------------------------- */

/* Probability of |1> on position pos (sum of |amp|^2 over indices with that bit set) for
 * 2^num_qubits amplitudes at device_amps, written to *device_result (device memory),
 * queued on stream (NULL = legacy default stream); returns without waiting.
 * No counterpart in the reference: this is iqsg_probability for callers that cannot
 * allocate device memory at that point (HBM already full, no implicit device-wide
 * synchronisation allowed, or a framework that owns all device memory). It calls no
 * cudaMalloc / cudaFree: its partial sums live in a static 16 KiB device array (2048
 * doubles) that every GPU loading the library keeps until exit. The first call on each
 * device looks that array up and should come before any stream capture. All calls share
 * the array, so calls that overlap on the GPU race. Sizes it cannot serve (num_qubits > 40,
 * or more than 2048 first-pass blocks) are rejected with IQSG_EINVAL. */
int iqsg_probability_static(const void* device_amps, unsigned num_qubits, int precision, unsigned pos,
                            double* device_result, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* IQSG_H */
