/*
 * tn_mps.h -- C ABI of the GB300 Schmidt-form (Gamma-Lambda) MPS trajectory engine.
 *
 * Drop-in boundary for whooie/tensor-net's `MPS<Q, C64>` trajectory path
 * (tensor-net/lib/mps.rs).  The reference is Rust and has no FFI of its own; the
 * entry points below are what a Rust `extern "C"` binding of that API binds,
 * one per inherent method it replaces (file:line cited beside each).
 *
 * Conventions (mirroring the reference):
 *  - complex numbers cross the ABI as interleaved (re, im) float64 pairs;
 *    matrices are row-major, so a 4x4 gate is 32 doubles, a 2x2 gate 8;
 *  - an out-of-range site/bond is a silent no-op for mutators (TN_OK) and
 *    TN_NONE for queries, as the reference returns `Ok(self)` / `None`;
 *  - a wrongly shaped operator is TN_ERR_OPERATOR_SHAPE (MPSError::
 *    OperatorIncompatibleShape, mps.rs:148-150);
 *  - randomness is never drawn inside the library: measurements take a
 *    caller-supplied uniform u in [0,1) in place of the reference's `rng.gen()`
 *    (mps.rs:1433); outcome = first s with u < cumsum(p)_s, i.e. (u < p0) ? 0 : 1;
 *  - one handle is one CUDA stream and is not thread-safe (the reference takes
 *    `&mut self`); distinct handles may be used from distinct threads;
 *  - host arrays passed in are read/written only during the call.
 *
 * Device state lives in HBM for the handle's lifetime: Gamma tensors in
 * fixed-capacity slots, Lambda vectors in float64, bond dimensions on the
 * device (truncation is decided on the GPU with no host round trip).
 */
#ifndef TN_MPS_H
#define TN_MPS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes (MPSError, mps.rs:126-154, plus device-side errors) ---- */
enum {
    TN_OK = 0,
    TN_NONE = 1,                     /* reference returns None (out-of-range query) */
    TN_CANCELLED = 2,                /* tn_result.status of a request ended by tn_server_cancel */
    TN_ERR_EMPTY_SYSTEM = -1,        /* MPSError::EmptySystem            mps.rs:131 */
    TN_ERR_INVALID_QNUM = -2,        /* MPSError::InvalidQuantumNumber   mps.rs:136 */
    TN_ERR_UNPHYSICAL_INDEX = -3,    /* MPSError::UnphysicalIndex        mps.rs:141 */
    TN_ERR_STATE_SHAPE = -4,         /* MPSError::StateIncompatibleShape mps.rs:146 */
    TN_ERR_OPERATOR_SHAPE = -5,      /* MPSError::OperatorIncompatibleShape mps.rs:150 */
    TN_ERR_INVALID_ARG = -6,         /* null pointer, bad enum, bad size */
    TN_ERR_CUDA = -7,                /* a CUDA runtime call failed */
    TN_ERR_OOM = -8,                 /* device or pinned-host allocation failed */
    TN_ERR_CAPACITY = -9,            /* a bond would exceed the handle's chi capacity */
    TN_ERR_NOT_CONVERGED = -10,      /* Jacobi SVD hit its sweep limit */
    TN_ERR_PROB_SUM = -11,           /* |p0 + p1 - 1| above tolerance at a measurement */
    TN_ERR_NO_DEVICE = -12           /* no CUDA device / kernels cannot run */
};

/* Truncation rule.  mps.rs:157-166 `BondDim` is Const(r) or Cutoff(eps);
 * `trunc = NULL` is the reference's `None` (cutoff at f64::EPSILON).
 * TN_TRUNC_BOTH is the combined rule used by the benchmark workloads:
 * rank = max(1, min(chi_max, #{leading s_j normal and > |cutoff|})). */
typedef enum {
    TN_TRUNC_NONE = 0,
    TN_TRUNC_CONST = 1,
    TN_TRUNC_CUTOFF = 2,
    TN_TRUNC_BOTH = 3
} tn_trunc_mode;

typedef struct {
    int32_t mode;       /* tn_trunc_mode */
    uint32_t chi_max;   /* CONST / BOTH */
    double cutoff;      /* CUTOFF / BOTH */
} tn_trunc;

/* Arithmetic of the device path.  F64: complex128 Gamma, float64 Jacobi SVD
 * (the plain path).  MIXED: complex64 Gamma and theta, float32 Jacobi sweeps
 * accumulated in float32, float64 Lambda, renormalisation, rank decision,
 * probabilities and entropies.  DF: FP64-class results on the FP32 pipes --
 * Gamma, theta and the Jacobi SVD in double-float arithmetic (pairs of float32,
 * about 48 significant bits), float64 Lambda, renormalisation, rank decision,
 * probabilities and entropies; the same 16 bytes per complex value as F64. */
typedef enum {
    TN_PREC_F64 = 0,
    TN_PREC_MIXED = 1,
    TN_PREC_DF = 2
} tn_precision;

typedef struct tn_mps tn_mps;
typedef struct tn_batch tn_batch;

const char *tn_status_string(int status);
/* Text of the last CUDA failure seen by the calling thread ("" if none). */
const char *tn_last_error(void);

/* Library / device information.  Fills `name` (cap bytes) with the GPU name and
 * `sm_count` with its SM count; TN_ERR_NO_DEVICE without a GPU. */
int tn_device_info(char *name, uint32_t cap, uint32_t *sm_count);

/* ======================= single state: MPS<Q, C64> ======================= */

/* MPS::new_qubits(n, trunc) (mps.rs:2033-2039 -> MPS::new, mps.rs:370-391):
 * |0...0>, every Gamma 1x2x1 with [0,0,0] = 1, every Lambda = [1].
 * chi_cap bounds every bond dimension (device slot size); 0 picks chi_max for
 * CONST/BOTH, else min(2^(n/2), 256).  n == 0 -> TN_ERR_EMPTY_SYSTEM. */
int tn_mps_new_qubits(uint32_t n, const tn_trunc *trunc, int32_t precision,
                      uint32_t chi_cap, tn_mps **out);
int tn_mps_free(tn_mps *m);
/* MPS::from_vector over qubits (mps.rs:517-550, factorize mps.rs:448-505):
 * state = 2^n interleaved complex128 amplitudes (s_0 most significant), len =
 * number of amplitudes.  Normalised, then factorised left to right on the
 * device (float64 one-sided Jacobi SVD per site, process_svd's rank rule with
 * `trunc`, NULL = Cutoff(f64::EPSILON)).  chi_cap 0 picks chi_max for
 * CONST/BOTH, else 2^(n/2).  n == 0 -> TN_ERR_EMPTY_SYSTEM; len != 2^n ->
 * TN_ERR_STATE_SHAPE; n > 20, a NULL state or a zero / non-finite norm ->
 * TN_ERR_INVALID_ARG. */
int tn_mps_from_vector(uint32_t n, const double *state, uint64_t len,
                       const tn_trunc *trunc, int32_t precision,
                       uint32_t chi_cap, tn_mps **out);
/* Checkpoint / resume: a state from its parts in the reference layout, the
 * inverse of tn_mps_export_gamma + tn_mps_svals (the reference has no
 * serialisation of MPS, mps.rs:338).  chi[n + 1] are the bond dimensions
 * with chi[0] = chi[n] = 1; gammas = Gamma_0 .. Gamma_{n-1} concatenated, each
 * (chi[k], 2, chi[k + 1]) row-major interleaved complex128; lams =
 * Lambda_0 .. Lambda_{n-2} concatenated (chi[1] .. chi[n-1] values).  The
 * parts are taken as they are (a state exported from a handle resumes
 * bit for bit in the same precision).  chi_cap 0 picks the larger of the
 * widest bond and the tn_mps_new_qubits rule.  chi[0] or chi[n] != 1 or a
 * zero bond -> TN_ERR_STATE_SHAPE; a bond above chi_cap -> TN_ERR_CAPACITY;
 * non-finite entries -> TN_ERR_INVALID_ARG. */
int tn_mps_import(uint32_t n, const uint32_t *chi, const double *gammas,
                  const double *lams, const tn_trunc *trunc, int32_t precision,
                  uint32_t chi_cap, tn_mps **out);
/* #[derive(Clone)] (mps.rs:338). */
int tn_mps_clone(const tn_mps *m, tn_mps **out);
int tn_mps_n(const tn_mps *m, uint32_t *n);
/* The handle's tn_precision. */
int tn_mps_precision(const tn_mps *m, int32_t *precision);
/* get_trunc / set_trunc (mps.rs:1216-1221); set_trunc(NULL) = None. */
int tn_mps_get_trunc(const tn_mps *m, tn_trunc *out);
int tn_mps_set_trunc(tn_mps *m, const tn_trunc *trunc);

/* apply_unitary1 (mps.rs:1298-1314): op is rows x cols complex, must be 2x2. */
int tn_mps_apply_unitary1(tn_mps *m, uint32_t k, const double *op,
                          uint32_t rows, uint32_t cols);
/* apply_unitary2 (mps.rs:1332-1387): op is rows x cols complex, must be 4x4,
 * acting on the fused pair index s_k*2 + s_{k+1}. */
int tn_mps_apply_unitary2(tn_mps *m, uint32_t k, const double *op,
                          uint32_t rows, uint32_t cols);

/* apply_unitary2 without any device allocation.  No counterpart in the
 * reference: for callers that cannot allocate device memory when they apply
 * a gate (a fixed memory plan that forbids allocation after start-up, or
 * work around a CUDA graph capture).  Same arguments and result as
 * tn_mps_apply_unitary2 (a non-finite gate entry is TN_ERR_INVALID_ARG);
 * the bond operation's scratch is a fixed 4.5 MiB device array shared by
 * every call: handles with a chi capacity above 270 in mixed precision or
 * above 191 in float64 / double-float are rejected with TN_ERR_CAPACITY.
 * Calls that overlap on the GPU race on that array: order them on one
 * stream.  The gate is staged from host memory during the call, so the
 * handle's stream must not be capturing (TN_ERR_INVALID_ARG).  The first
 * call on a device looks up the array's address; make it before any stream
 * capture begins. */
int tn_mps_apply_unitary2_noalloc(tn_mps *m, uint32_t k, const double *op,
                                  uint32_t rows, uint32_t cols);

/* probs (mps.rs:1071-1076): out[0..2]. */
int tn_mps_probs(const tn_mps *m, uint32_t k, double out[2]);
/* prob (mps.rs:1138-1143). */
int tn_mps_prob(const tn_mps *m, uint32_t k, uint32_t p, double *out);

/* measure_prob (mps.rs:1479-1489): sample with uniform u, project, full
 * refactor sweep (mps.rs:894-897). */
int tn_mps_measure_prob(tn_mps *m, uint32_t k, double u,
                        int32_t *outcome, double *prob);
/* measure_postsel_prob (mps.rs:1501-1510). */
int tn_mps_measure_postsel_prob(tn_mps *m, uint32_t k, uint32_t p, double *prob);

/* apply_meas_prob_layer (mps.rs:2206-2252) / measure_prob_layer (1552-1582).
 * ks[nk] targets in any order; out-of-range ones are dropped, duplicates
 * removed (first kept), the rest sorted ascending.  `posts` may be NULL (all
 * Meas::Rand); posts[i] >= 0 makes target i a Meas::Proj post-selection.
 * us[j] is the uniform of the j-th surviving target in ascending order (the
 * order the reference draws from its rng).  Outputs (capacity nk each):
 * out_ks, outcomes, probs; *n_out = number of surviving targets. */
int tn_mps_apply_meas_prob_layer(tn_mps *m, const uint32_t *ks, uint32_t nk,
                                 const int32_t *posts, const double *us,
                                 uint32_t *out_ks, int32_t *outcomes, double *probs,
                                 uint32_t *n_out);

/* circuit::apply_bilayer (circuit.rs:624-659) with Uni::Mat 4x4 gates:
 * gates[ng*32] applied at gate_ks[ng] in order (apply_unitary2), then one
 * apply_meas_prob_layer over meas_ks/us (posts NULL).  One device launch. */
int tn_mps_apply_bilayer(tn_mps *m, const uint32_t *gate_ks, const double *gates,
                         uint32_t ng, const uint32_t *meas_ks, uint32_t nm,
                         const double *us, uint32_t *out_ks, int32_t *outcomes,
                         double *probs, uint32_t *n_out);

/* entropy_vn (mps.rs:1251-1261), float64 on the device. */
int tn_mps_entropy_vn(const tn_mps *m, uint32_t b, double *out);
/* entropy_ry_schmidt (mps.rs:1268-1282). */
int tn_mps_entropy_ry_schmidt(const tn_mps *m, double a, uint32_t b, double *out);
/* bond_dim / max_bond_dim (mps.rs:1224-1245). */
int tn_mps_bond_dim(const tn_mps *m, uint32_t b, uint32_t *out);
int tn_mps_max_bond_dim(const tn_mps *m, uint32_t *out);
/* Lambda on bond b (the reference's svals[b], mps.rs:352-353). */
int tn_mps_svals(const tn_mps *m, uint32_t b, double *out, uint32_t cap, uint32_t *len);
/* Gamma of site k in the reference layout (chi_{k-1}, 2, chi_k), row-major,
 * interleaved complex128 (mps.rs:344-349).  dims[3] receives the shape. */
int tn_mps_export_gamma(const tn_mps *m, uint32_t k, double *out, uint64_t cap,
                        uint32_t dims[3]);
/* contract (mps.rs:794-798): the dense 2^n state vector, interleaved
 * complex128, s_0 most significant; n <= 24. */
int tn_mps_contract(const tn_mps *m, double *out, uint64_t cap);
/* Device-side error word accumulated by this handle's kernels (0 if none);
 * cleared on read. */
int tn_mps_device_status(tn_mps *m, int32_t *status);
/* Work counters accumulated on the device since the last reset, 16 doubles:
 * [0] theta flops 8*(2chiL)*chiM*(2chiR) (+128*chiL*chiR per gate),
 * [1] SVD flops 4*(4a^2b + 8ab^2 + 9b^3) (a, b = larger/smaller side of theta),
 * [2] bond operations, [3] Jacobi sweeps, [4] measurements,
 * [5] algorithmic HBM bytes, [6..10] SM cycles spent in theta build, block
 * Gram, block rotations, block update and finalisation, [11] Jacobi block
 * steps, [12] refactors done through the LQ-reduced matrix, [13] SVDs that hit
 * the sweep limit, [14]/[15] sum of their vector counts (LQ / direct path).  reset != 0 zeroes them. */
int tn_mps_stats(tn_mps *m, double *out, int32_t reset);

/* ==================== batch of trajectories (batching) ==================== */

/* Many independent trajectories, each its own MPS (own n, truncation), all
 * resident on the device; one persistent launch advances every active
 * trajectory by one brickwork layer (gates, measurement layer with its
 * refactor sweep, half-chain entropy).  Results per trajectory do not depend
 * on which other trajectories share the launch. */
int tn_batch_create(uint32_t ntraj, const uint32_t *ns, const tn_trunc *truncs,
                    int32_t precision, const uint32_t *chi_caps, tn_batch **out);
int tn_batch_free(tn_batch *b);
/* Re-initialise slot t to |0...0> with a new n/trunc (n and chi must fit the
 * slot's allocation); used by the serving loop to reuse slots. */
int tn_batch_reset(tn_batch *b, uint32_t t, uint32_t n, const tn_trunc *trunc);
/* Slot t := a state given by its reference-layout parts (as tn_mps_import:
 * chi[n + 1], Gamma_0 .. Gamma_{n-1} and Lambda_0 .. Lambda_{n-2}
 * concatenated), with truncation rule `trunc`: a prepared initial state
 * (tn_mps_from_vector) or a checkpoint enters the batch.  n up to the slot's
 * allocated n, every bond up to the slot's bond capacity (TN_ERR_CAPACITY). */
int tn_batch_import(tn_batch *b, uint32_t t, uint32_t n, const uint32_t *chi,
                    const double *gammas, const double *lams, const tn_trunc *trunc);
/* Gamma of site k of slot t in the reference layout (as tn_mps_export_gamma). */
int tn_batch_export_gamma(tn_batch *b, uint32_t t, uint32_t k, double *out,
                          uint64_t cap, uint32_t dims[3]);

/* One brickwork layer for the trajectories listed in `trajs[nt]`:
 * trajectory trajs[i] applies gates gate_off[i]..gate_off[i+1]-1 (sites
 * gate_ks[], 4x4 complex128 gates[32 each]) then measures sites
 * meas_off[i]..meas_off[i+1]-1 (meas_ks[] sorted ascending, unique, in range;
 * uniforms us[]).  Outputs: outcomes[]/probs[] parallel to meas_ks, and
 * entropy[i] = entropy_vn(n/2 - 1) after the layer.  Host arrays; the call
 * copies them in, launches once, copies results back and synchronises. */
int tn_batch_step(tn_batch *b, const uint32_t *trajs, uint32_t nt,
                  const uint32_t *gate_off, const uint32_t *gate_ks, const double *gates,
                  const uint32_t *meas_off, const uint32_t *meas_ks, const double *us,
                  int32_t *outcomes, double *probs, double *entropy);

/* tn_batch_step with post-selection: posts[j] (parallel to meas_ks) = 0 or 1
 * projects site meas_ks[j] onto that outcome and reports its Born
 * probability (Meas::Proj in apply_meas_prob_layer, mps.rs:2236-2242; its
 * uniform is unused), any other value samples with us[j] (Meas::Rand).
 * posts = NULL is tn_batch_step. */
int tn_batch_step_post(tn_batch *b, const uint32_t *trajs, uint32_t nt,
                       const uint32_t *gate_off, const uint32_t *gate_ks, const double *gates,
                       const uint32_t *meas_off, const uint32_t *meas_ks, const double *us,
                       const int32_t *posts, int32_t *outcomes, double *probs, double *entropy);

/* Same layer, inputs already in device memory (pointers from tn_batch_device_inputs);
 * no host copies, no synchronisation (stream-ordered on the batch stream). */
int tn_batch_device_inputs(tn_batch *b, uint32_t max_gates, uint32_t max_meas,
                           void **d_trajs, void **d_gate_off, void **d_gate_ks,
                           void **d_gates, void **d_meas_off, void **d_meas_ks,
                           void **d_us, void **d_outcomes, void **d_probs,
                           void **d_entropy);
int tn_batch_step_device(tn_batch *b, uint32_t nt);
/* Same layer with every array supplied by the caller in device memory
 * (int32 indices, float64 gates/uniforms): trajs[nt], order[nt] (execution
 * rank of each entry: a permutation of 0..nt-1, 0 runs first; NULL = most
 * expensive first by the current bond dimensions, ranked on the device), gate_off[nt+1],
 * gate_ks[], gates[32 per gate], meas_off[nt+1], meas_ks[], us[], and outputs
 * outcomes[], probs[], entropy[nt].  Stream-ordered on the batch stream, no
 * synchronisation, no host copies. */
int tn_batch_step_ptrs(tn_batch *b, uint32_t nt, const void *d_trajs, const void *d_order,
                       const void *d_gate_off, const void *d_gate_ks, const void *d_gates,
                       const void *d_meas_off, const void *d_meas_ks, const void *d_us,
                       void *d_outcomes, void *d_probs, void *d_entropy);
int tn_batch_synchronize(tn_batch *b);
/* Per-trajectory queries (same meaning as the tn_mps_* ones). */
int tn_batch_bond_dims(tn_batch *b, uint32_t t, uint32_t *out, uint32_t cap);
int tn_batch_svals(tn_batch *b, uint32_t t, uint32_t bond, double *out, uint32_t cap,
                   uint32_t *len);
/* Or of the device error words of every trajectory (bits: 1 SVD sweep limit
 * hit, 2 capacity, 4 probability sum, 8 bad instruction list) and 16 when a
 * CTA's wait for a pushed work item ran past its limit; cleared on read. */
int tn_batch_device_status(tn_batch *b, int32_t *status);
/* Sum of the work counters (see tn_mps_stats) over all trajectories. */
int tn_batch_stats(tn_batch *b, double *out, int32_t reset);
/* Device bytes held by slot t (its footprint for admission control). */
int tn_batch_slot_bytes(tn_batch *b, uint32_t t, uint64_t *bytes);
/* theta contraction of the mixed-precision executor: 0 (default) tensor
 * cores (tcgen05, 3xTF32) where the tile shape applies, 1 the SIMT FP32
 * contraction everywhere.  No counterpart in the reference. */
int tn_batch_set_theta_path(tn_batch *b, int32_t simt);
/* Online autotuner: the next 4 * trial_steps host- or pointer-launched steps
 * (tn_batch_step, tn_batch_step_ptrs) run, trial_steps each, the candidate
 * configurations {schedule 1, Jacobi scheme 3, tensor-core theta},
 * {1, 0, tensor-core}, {0, 3, tensor-core}, {1, 3, SIMT theta}; each is
 * scored by device launch time per algorithmic flop (device counters), and
 * the best is kept (captured graphs are re-captured with it).  trial_steps
 * = 0 stops tuning.  Results are the same under every candidate up to the
 * rounding of the chosen arithmetic.  No counterpart in the reference. */
int tn_batch_autotune(tn_batch *b, uint32_t trial_steps);
/* cfg[4]: schedule, Jacobi scheme, SIMT theta (1) / tensor-core theta (0),
 * tuning in progress; scores[4] (may be NULL): seconds per flop per candidate. */
int tn_batch_tuning(tn_batch *b, int32_t *cfg, double *scores);
/* Schedule of a layer step: 1 (default) = one persistent launch in which
 * every gate of the layer is a work item and a trajectory's measurement
 * layer, refactor sweep and entropy read become a work item as soon as its
 * last gate item has finished; 0 = two launches (all gate items, then all
 * sweep programs).  Results are bit-identical; 1 removes the idle time of the
 * barrier between the two phases.  No counterpart in the reference. */
int tn_batch_set_schedule(tn_batch *b, int32_t schedule);
/* Jacobi tuning of the batch (picked by the autotuner): scheme 0 visits all
 * vector pairs of each block pair of a sweep, scheme 1 visits every pair once
 * per sweep (within-block steps, then cross-block steps), scheme 2 / 3 is
 * scheme 0 with two inner sweeps per block step during the first two / three
 * sweeps (default 3); max_sweeps bounds the sweeps of one SVD (1..200,
 * default 40). */
int tn_batch_set_tuning(tn_batch *b, int32_t scheme, int32_t max_sweeps);
/* Device time of the last non-graph step, split into the gate launch (all
 * gates of the layer as independent items) and the sweep launch (measurement
 * layers, refactor sweeps, entropy reads).  TN_NONE before any such step. */
int tn_batch_last_launch_ms(tn_batch *b, float *gate_ms, float *sweep_ms);
/* Device time (CUDA events on the batch stream) of the last tn_batch_step /
 * tn_batch_step_post call from the end of its input copy to the start of its
 * output copy: every kernel of the layer, with its inputs resident in HBM.
 * TN_NONE before the first such step. */
int tn_batch_last_step_device_ms(tn_batch *b, float *ms);
/* Failure detection of the one-launch schedule (no counterpart in the
 * reference).  A CTA that has claimed a sweep slot waits for the item to be
 * pushed at most wait_ns nanoseconds (0 = the default, 120 s); past it, the
 * CTA sets ST_QUEUE_WAIT (bit 16 of tn_batch_device_status) and moves on, so
 * the launch always ends.  phantom_sweeps adds sweep slots that no work item
 * ever fills (capped by the step buffers' trajectory capacity), which makes
 * the wait run out on purpose: a test of the limit and of the error report.
 * Both settings hold for later steps until changed. */
int tn_batch_set_queue_wait(tn_batch *b, uint64_t wait_ns, uint32_t phantom_sweeps);
/* Stream the batch launches on (a cudaStream_t), for callers that time with
 * CUDA events. */
int tn_batch_stream(tn_batch *b, void **stream);

/* ================= serving: continuous batching of requests ================= */

/* One trajectory request: a seeded Haar brickwork trajectory (inputs from
 * tn_gen_layer(seed, traj, layer, n, p)) of `depth` layers from |0...0>. */
typedef struct {
    uint32_t n;
    tn_trunc trunc;
    double p;
    uint32_t depth;
    uint64_t seed;
    uint64_t traj;
} tn_request;

typedef struct {
    uint64_t id;
    uint32_t layers;
    double final_entropy;  /* entropy_vn(n/2 - 1) after the last layer */
    double latency_s;      /* completion - arrival, server clock */
    double queue_s;        /* admission - arrival */
    int32_t status;
} tn_result;

typedef struct tn_server tn_server;

/* A server with an HBM arena of hbm_bytes for request state, up to max_slots
 * requests resident at once per cost class, requests up to max_n qubits and
 * bond capacity max_chi.  Admission (first come, first served within a class)
 * needs a free slot and the request's projected footprint
 * n * cap^2 * 2 complex values + Lambdas in the arena.  Requests with bond
 * capacity <= light_chi form class 0, the rest class 1; each class advances
 * its admitted requests one layer per persistent launch on its own stream and
 * share of the SMs (light_ctas CTAs for class 0, the remaining SMs for class
 * 1), independently of the other class, and retires finished requests,
 * freeing their memory.  light_chi = 0 means 64, light_ctas = 0 means a fifth
 * of the SMs; light_chi >= max_chi gives one class over every SM.  No
 * counterpart in the reference (which runs trajectories one per thread,
 * workspace/src/haar_coev_probs.rs:164). */
int tn_server_create_classes(uint64_t hbm_bytes, uint32_t max_slots, int32_t precision,
                             uint32_t max_chi, uint32_t max_n, uint32_t light_chi,
                             uint32_t light_ctas, tn_server **out);
/* tn_server_create_classes with the default classes. */
int tn_server_create(uint64_t hbm_bytes, uint32_t max_slots, int32_t precision,
                     uint32_t max_chi, uint32_t max_n, tn_server **out);
int tn_server_free(tn_server *s);
/* Seconds since the server was created (the clock of arrivals and latencies). */
int tn_server_now(const tn_server *s, double *t);
/* Queue a request; arrival < 0 means now.  TN_ERR_CAPACITY if it can never fit. */
int tn_server_submit(tn_server *s, const tn_request *r, double arrival, uint64_t *id);
/* Launch the next layer of every idle class (after admitting what fits),
 * wait until at least one class has finished its layer, retire the requests
 * of that class that reached their depth and relaunch it.  n_active = requests
 * resident after the tick, n_done = requests retired by it. */
int tn_server_tick(tn_server *s, uint32_t *n_active, uint32_t *n_done);
/* Completed requests (up to cap). */
int tn_server_poll(tn_server *s, tn_result *out, uint32_t cap, uint32_t *n);
/* Half-chain entropy after every layer of retired request `id` (the
 * reference's per-trajectory output, entropy_vn(n/2 - 1) per layer), in
 * layer order; *len = layers run.  With out = NULL only *len is set; a
 * successful copy releases the record (each retired request's record is kept
 * until fetched or the server is freed).  TN_NONE for an unknown or already
 * fetched id. */
int tn_server_history(tn_server *s, uint64_t id, double *out, uint32_t cap, uint32_t *len);
/* Cancel request `id`.  A queued request is dropped at once; a resident one
 * is retired when the layer it is part of finishes (no kernel of the server
 * is using its memory after that), its slot and arena range freed.  Either
 * way a tn_result with status TN_CANCELLED and the layers completed so far
 * is queued for tn_server_poll.  TN_NONE if the id is unknown or already
 * finished. */
int tn_server_cancel(tn_server *s, uint64_t id);
/* [0] traj-layers run, [1] seconds inside ticks, [2] ticks, [3] arena bytes in
 * use, [4] pending, [5] active, [6] admitted, [7] completed. */
int tn_server_stats(const tn_server *s, double *out);
/* Admission policy within each class: 0 (default) first come, first served;
 * 1 least estimated work first (depth * n * cap^3).  max_active0/1 bound the
 * requests resident in class 0/1 at once (0 = every slot), which bounds the
 * time of one layer launch of that class and so the service time of each
 * admitted request. */
int tn_server_set_policy(tn_server *s, int32_t policy, uint32_t max_active0, uint32_t max_active1);
/* Class cls (0 or 1): [0] bond capacity bound, [1] CTA limit (0 = all),
 * [2] traj-layers run, [3] launches, [4] pending, [5] active; zeros for a
 * class the server does not have. */
int tn_server_class_stats(const tn_server *s, uint32_t cls, double *out);

/* ======================= seeded synthetic inputs ======================= */

/* gate::haar(2, rng) (gate.rs:888-909) given the Ginibre sample z (4x4
 * complex128, row-major, interleaved): QR, then column j divided by
 * r_jj/|r_jj|.  Host code, float64. */
int tn_haar_u4(const double *z, double *out);

/* Counter-based generator of one brickwork layer of one trajectory
 * (circuit.rs:558-584 haar_layer + uniform_meas, gate positions
 * workspace/lib/haar.rs:285: offset = layer odd): all values are pure
 * functions of (seed, traj, layer, site, purpose).  gates[] needs room for
 * 32*(n/2) doubles, gate_ks/meas_ks/us for n entries.  Host code. */
int tn_gen_layer(uint64_t seed, uint64_t traj, uint32_t layer, uint32_t n, double p,
                 uint32_t *gate_ks, double *gates, uint32_t *ng,
                 uint32_t *meas_ks, double *us, uint32_t *nm);

/* The Ginibre sample (4x4 complex128) behind the gate at `site` of a layer
 * produced by tn_gen_layer, for checking tn_haar_u4 against another QR. */
int tn_gen_ginibre(uint64_t seed, uint64_t traj, uint32_t layer, uint32_t site, double *z);

#ifdef __cplusplus
}
#endif

#endif /* TN_MPS_H */
