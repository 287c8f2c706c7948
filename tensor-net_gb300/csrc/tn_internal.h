// tn_internal.h -- types shared by the host runtime and the kernels.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace tn {

// Threads per executor CTA and Jacobi block-pair width.
constexpr int kThreads = 512;
constexpr int kBlockW = 32;

// Instruction set of a trajectory program (one CTA executes one program).
enum Opcode : int {
  OP_NOP = 0,
  OP_GATE = 1,      // k, a = gate index          apply_unitary2 (mps.rs:1332)
  OP_REFACTOR = 2,  // k                          local_refactor (mps.rs:846)
  OP_MEAS = 3,      // k, a = slot, b = post|-1   sample_state+project (mps.rs:1427-1465)
  OP_ENTROPY = 4,   // k = bond, a = slot         entropy_vn (mps.rs:1251)
  OP_UNI1 = 5,      // k, a = gate index          apply_unitary1 (mps.rs:1298)
  OP_PROBS = 6,     // k, a = slot                local_probs (mps.rs:1079)
  OP_RENYI = 7      // k = bond, a = slot, b = index of alpha in us[]  entropy_ry_schmidt (mps.rs:1268)
};

struct Instr {
  int op, k, a, b;
};

// Device error word bits (or-ed into *TrajDev::status).
enum : int {
  ST_NOT_CONVERGED = 1,
  ST_CAPACITY = 2,
  ST_PROB_SUM = 4,
  ST_BAD_INSTR = 8,
  ST_QUEUE_WAIT = 16,  // a CTA's wait for a pushed work item ran past its limit (batch-wide)
};

// Per-trajectory counters accumulated by the kernels (float64 slots).
enum : int {
  STAT_FLOP_THETA = 0,  // 8*(2chiL)*chiM*(2chiR) (+128*chiL*chiR for a gate)
  STAT_FLOP_SVD = 1,    // 4*(4a^2 b + 8ab^2 + 9b^3), a/b = max/min(2chiL, 2chiR)
  STAT_BOND_OPS = 2,
  STAT_SWEEPS = 3,
  STAT_MEAS = 4,
  STAT_BYTES = 5,       // algorithmic HBM bytes of the bond ops and measurements
  STAT_CYC_THETA = 6,   // SM cycles (thread 0 clock64) per phase of the bond operations
  STAT_CYC_GRAM = 7,
  STAT_CYC_ROT = 8,     // inner Jacobi on the block Gram matrix
  STAT_CYC_UPDATE = 9,
  STAT_CYC_FINAL = 10,
  STAT_BLOCK_STEPS = 11,
  STAT_LQ_OPS = 12,     // refactors done through the LQ-reduced matrix
  STAT_NONCONV = 13,    // Jacobi SVDs that hit the sweep limit
  STAT_NONCONV_LQ = 14,      // sum of their vector counts, LQ path
  STAT_NONCONV_DIRECT = 15,  // sum of their vector counts, direct path
  STAT_N = 16
};

struct TrajDev {
  void *gamma;     // n slots of 2*cap*cap complex<T>
  double *lam;     // n+1 slots of cap float64
  int *chi;        // n+1 bond dimensions (chi[0] = chi[n] = 1)
  int *status;     // error word
  double *stats;   // STAT_N counters
  int n, cap;
  int trunc_mode, chi_max;
  double cutoff;
};

// A work item: `len` instructions from `off` of a program array, on slot
// `traj`.  aux: for a gate item of the dependency-driven schedule, the list
// index of its trajectory; for a pushed sweep slot, 1 once it is written.
struct Item {
  int traj, off, len, aux;
};

struct LaunchArgs {
  const Item *items;
  int nitems;
  const int *nitems_dev;  // when set, the item count is read from device memory
  int *counter;
  TrajDev *trajs;
  const Instr *prog;
  const double *gates;   // 32 doubles per gate (4x4 complex128 row-major)
  const double *us;      // uniforms (and Renyi alphas)
  int *outcomes;
  double *probs;
  double *ents;
  double *pout;          // OP_PROBS output, 2 per slot
  void *ws;              // per-CTA workspace
  size_t ws_stride;      // bytes per CTA
  int max_sweeps;
  int jacobi_scheme;      // 0: block pairs, all pairs per step; 1: within-block then cross-block steps
  int theta_simt;         // 1: SIMT theta contraction even where the tensor-core one applies
  // Dependency-driven schedule (rem != nullptr): items[0, *nitems_dev) are
  // gate items with programs in gprog; when the last gate item of listed
  // trajectory i finishes, its sweep item sweeps[i] is pushed to dyn, and the
  // queue continues with those pushed items (nsweeps of them) in push order.
  const Instr *gprog;
  int *rem;               // per listed trajectory: gate items not yet finished
  const Item *sweeps;     // per listed trajectory: measurement layer + sweep + entropy program
  Item *dyn;              // pushed sweep items (aux = 1 once written); zeroed before compile
  int *dyn_tail;          // push counter; zeroed before compile
  int *dyn_head;          // sweep slots claimed; zeroed before the launch
  int nsweeps;
  int *qerr;              // set to 1 when a queue wait ran past its time limit
  unsigned long long queue_wait_ns;  // limit of one such wait (0: kQueueWaitNs)
};

// Default Jacobi block scheme (see jacobi_svd): all pairs of each block pair,
// two inner sweeps per step during the first three sweeps.
constexpr int kDefaultScheme = 3;

// Wait limit of a CTA on a pushed queue slot (nanoseconds of %globaltimer).
constexpr unsigned long long kQueueWaitNs = 120ull * 1000 * 1000 * 1000;

cudaError_t launch_run(int prec, const LaunchArgs &la, int grid, int sortP, int ws_cap, cudaStream_t st);
size_t run_smem_bytes(int prec, int sortP);
size_t run_work_bytes(int prec, int cap);
int run_blocks_per_sm(int prec, int sortP);
cudaError_t launch_reset(TrajDev *trajs, const int *list, int count, int prec, cudaStream_t st);
// posts (may be null): per measurement, 0 / 1 = post-selected outcome (Meas::Proj), else sampled
cudaError_t launch_compile(const TrajDev *trajs, const int *list, int nt, const int *order, const int *gate_off,
                           const int *gate_ks, const int *meas_off, const int *meas_ks, const int *posts, int pcap,
                           Instr *prog, Item *items, Instr *gprog, Item *gitems, int gcap, int *gcount,
                           cudaStream_t st);
// order[i] = execution rank of listed trajectory i, most expensive first by
// the current bond dimensions (a single-block sort on the device).
cudaError_t launch_lpt_order(const TrajDev *trajs, const int *list, int nt, const int *meas_off, int *order,
                             cudaStream_t st);
// Dependency-driven variant: gate items placed trajectory by trajectory in
// `order` rank (gstart from a scan over ranks, scratch: nt ints), sweep
// programs at sweeps[i], rem[i] = gate items of trajectory i, and trajectories
// without gate items pushed at once.
cudaError_t launch_compile_dd(const TrajDev *trajs, const int *list, int nt, const int *order, const int *gate_off,
                              const int *gate_ks, const int *meas_off, const int *meas_ks, const int *posts, int pcap,
                              Instr *prog, Item *sweeps, Instr *gprog, Item *gitems, int gcap, int *gcount,
                              int *gstart, int *scratch, int *rem, Item *dyn, int *dyn_tail, cudaStream_t st);

// Device-side view of a single-state handle (for entry points outside
// tn_host.cpp that launch on it).
struct MpsView {
  TrajDev *dtraj;
  int n, cap, prec;
  cudaStream_t st;
};
}  // namespace tn
struct tn_mps;
namespace tn {
int mps_view(const tn_mps *m, MpsView *out);

}  // namespace tn
struct tn_batch;
namespace tn {
// Engine mode of a batch (serving): slots bound to caller-managed memory.
tn_batch *batch_engine_create(uint32_t slots, int prec, int ws_cap, int max_n, int grid_limit, int *status);
int batch_step_collect(tn_batch *b, int32_t *outcomes, double *probs, double *entropy);
bool batch_step_done(tn_batch *b);
int batch_bind(tn_batch *b, uint32_t t, const TrajDev &d);
cudaStream_t batch_stream(tn_batch *b);

// Record the text of a failed CUDA call for tn_last_error() (thread-local).
void set_last_error(const char *what, cudaError_t e);

// Device element layout of a precision: F64 complex128 (16 bytes), MIXED
// complex64 (8 bytes), DF double-float complex (four floats re.hi, re.lo,
// im.hi, im.lo: 16 bytes).
inline size_t prec_elem_bytes(int prec) { return prec == 1 ? 8 : 16; }
// n real parts (interleaved complex128) to the device layout of prec (dst
// holds n * prec_elem_bytes(prec) / 2 bytes) and back.
inline void reals_to_layout(int prec, const double *src, size_t n, void *dst) {
  if (prec == 0) {
    for (size_t i = 0; i < n; ++i) static_cast<double *>(dst)[i] = src[i];
  } else if (prec == 2) {
    float *d = static_cast<float *>(dst);
    for (size_t i = 0; i < n; ++i) {
      const float hi = float(src[i]);
      d[2 * i] = hi;
      d[2 * i + 1] = float(src[i] - double(hi));
    }
  } else {
    for (size_t i = 0; i < n; ++i) static_cast<float *>(dst)[i] = float(src[i]);
  }
}
inline void layout_to_reals(int prec, const void *src, size_t n, double *dst) {
  if (prec == 0) {
    for (size_t i = 0; i < n; ++i) dst[i] = static_cast<const double *>(src)[i];
  } else if (prec == 2) {
    const float *s = static_cast<const float *>(src);
    for (size_t i = 0; i < n; ++i) dst[i] = double(s[2 * i]) + double(s[2 * i + 1]);
  } else {
    for (size_t i = 0; i < n; ++i) dst[i] = double(static_cast<const float *>(src)[i]);
  }
}

inline int next_pow2(int x) {
  int p = 1;
  while (p < x) p <<= 1;
  return p;
}

}  // namespace tn
