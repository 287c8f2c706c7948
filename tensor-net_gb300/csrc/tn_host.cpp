// tn_host.cpp -- host runtime behind include/tn_mps.h.
//
// Turns each reference API call into a short instruction list (the control
// flow of tensor-net/lib/mps.rs: sort/dedup of measurement targets, refactor
// ranges of the sweeps) and runs it with the persistent executor kernel on the
// handle's stream.  No host round trip is needed between operations: bond
// dimensions and truncation live on the device.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "tn_internal.h"
#include "tn_mps.h"

using namespace tn;

namespace {

thread_local std::string g_last_error;

}  // namespace

void tn::set_last_error(const char *what, cudaError_t e) {
  g_last_error = e == cudaSuccess ? std::string(what) : std::string(what) + ": " + cudaGetErrorString(e);
  // A failed call also becomes the runtime's "last error" of this thread; a
  // non-sticky one (a refused allocation) would otherwise be reported again
  // by the cudaGetLastError() after the next kernel launch.  Consume it.
  if (e != cudaSuccess) (void)cudaGetLastError();
}

namespace {

int cuda_fail(cudaError_t e, const char *what) {
  tn::set_last_error(what, e);
  if (e == cudaErrorMemoryAllocation) return TN_ERR_OOM;
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return TN_ERR_NO_DEVICE;
  return TN_ERR_CUDA;
}

#define CK(call)                                         \
  do {                                                   \
    cudaError_t e__ = (call);                            \
    if (e__ != cudaSuccess) return cuda_fail(e__, #call); \
  } while (0)

struct DevBuf {
  void *p = nullptr;
  size_t n = 0;
  cudaError_t ensure(size_t bytes) {
    if (bytes <= n) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
    size_t want = std::max<size_t>(bytes, 256);
    cudaError_t e = cudaMalloc(&p, want);
    if (e == cudaSuccess) n = want;
    return e;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  template <typename X>
  X *as() const {
    return reinterpret_cast<X *>(p);
  }
};

struct HostBuf {
  void *p = nullptr;
  size_t n = 0;
  cudaError_t ensure(size_t bytes) {
    if (bytes <= n) return cudaSuccess;
    if (p) cudaFreeHost(p);
    p = nullptr;
    n = 0;
    size_t want = std::max<size_t>(bytes, 256);
    cudaError_t e = cudaMallocHost(&p, want);
    if (e == cudaSuccess) n = want;
    return e;
  }
  void release() {
    if (p) cudaFreeHost(p);
    p = nullptr;
    n = 0;
  }
};

constexpr int kMaxSweeps = 40;

uint32_t max_schmidt_rank(uint32_t n) {
  uint32_t h = n / 2;
  if (h >= 20) return 1u << 20;
  return 1u << h;
}

uint32_t default_cap(uint32_t n, const tn_trunc *tr) {
  uint32_t lim = max_schmidt_rank(n);
  if (tr && (tr->mode == TN_TRUNC_CONST || tr->mode == TN_TRUNC_BOTH)) {
    uint32_t c = std::max<uint32_t>(1, tr->chi_max);
    return std::min(c, lim);
  }
  return std::min<uint32_t>(lim, 256);
}

int check_trunc(const tn_trunc *tr) {
  if (!tr) return TN_OK;
  if (tr->mode < TN_TRUNC_NONE || tr->mode > TN_TRUNC_BOTH) return TN_ERR_INVALID_ARG;
  return TN_OK;
}

void fill_trunc(TrajDev &d, const tn_trunc *tr) {
  if (!tr) {
    d.trunc_mode = TN_TRUNC_NONE;
    d.chi_max = 0;
    d.cutoff = 0.0;
  } else {
    d.trunc_mode = tr->mode;
    d.chi_max = int(std::min<uint32_t>(tr->chi_max, 0x7fffffff));
    d.cutoff = tr->cutoff;
  }
}

size_t elem_bytes(int prec) { return prec_elem_bytes(prec); }

// Host restatement of the measurement-layer control flow of
// apply_meas_prob_layer (mps.rs:2206-2252): targets already filtered, sorted,
// deduplicated; slot j of us/outcomes belongs to targets[j].
void emit_meas_layer(std::vector<Instr> &prog, uint32_t n, const std::vector<uint32_t> &targets,
                     const std::vector<int32_t> &posts, int slot0) {
  if (targets.empty()) return;
  int last = -1;
  for (size_t j = 0; j < targets.size(); ++j) {
    int k = int(targets[j]);
    if (last >= 0)
      for (int b = last; b < k; ++b) prog.push_back(Instr{OP_REFACTOR, b, 0, 0});
    prog.push_back(Instr{OP_MEAS, k, slot0 + int(j), posts.empty() ? -1 : posts[j]});
    last = k;
  }
  for (int b = last; b < int(n) - 1; ++b) prog.push_back(Instr{OP_REFACTOR, b, 0, 0});
  for (int b = int(n) - 3; b >= 0; --b) prog.push_back(Instr{OP_REFACTOR, b, 0, 0});
}

// refactor_sweep (mps.rs:894-897)
void emit_sweep(std::vector<Instr> &prog, uint32_t n) {
  for (int b = 0; b < int(n) - 1; ++b) prog.push_back(Instr{OP_REFACTOR, b, 0, 0});
  for (int b = int(n) - 3; b >= 0; --b) prog.push_back(Instr{OP_REFACTOR, b, 0, 0});
}

// Launch scratch shared by the single-state API calls of one handle.
struct Launcher {
  DevBuf prog, items, counter, gates, us, outc, probs, ents, pout, ws, gprog, gitems;
  int sortP = 1, ws_cap = 1, ws_ctas = 1, sms = 1;
  void release() {
    gprog.release();
    gitems.release();
    prog.release();
    items.release();
    counter.release();
    gates.release();
    us.release();
    outc.release();
    probs.release();
    ents.release();
    pout.release();
    ws.release();
  }
};

}  // namespace

// ====================================================================== tn_mps
struct tn_mps {
  uint32_t n = 0, cap = 1;
  int prec = TN_PREC_F64;
  bool has_trunc = false;
  tn_trunc trunc{};
  cudaStream_t st = nullptr;
  DevBuf gamma, lam, chi, status, dtraj, stats;
  TrajDev h{};
  Launcher L;
};

extern "C" {

const char *tn_status_string(int s) {
  switch (s) {
    case TN_OK: return "ok";
    case TN_NONE: return "none (out of range)";
    case TN_CANCELLED: return "cancelled";
    case TN_ERR_EMPTY_SYSTEM: return "error in MPS creation: cannot create for an empty system";
    case TN_ERR_INVALID_QNUM: return "error in MPS creation: invalid quantum number";
    case TN_ERR_UNPHYSICAL_INDEX: return "error in MPS creation: unphysical zero-dimensional physical index";
    case TN_ERR_STATE_SHAPE: return "error in MPS creation: array length/shape doesn't match indices";
    case TN_ERR_OPERATOR_SHAPE: return "error in operator application: incorrect shape";
    case TN_ERR_INVALID_ARG: return "invalid argument";
    case TN_ERR_CUDA: return "CUDA runtime error";
    case TN_ERR_OOM: return "out of memory";
    case TN_ERR_CAPACITY: return "bond dimension exceeds the handle's capacity";
    case TN_ERR_NOT_CONVERGED: return "Jacobi SVD did not converge within its sweep limit";
    case TN_ERR_PROB_SUM: return "outcome probabilities do not sum to one";
    case TN_ERR_NO_DEVICE: return "no CUDA device";
    default: return "unknown status";
  }
}

const char *tn_last_error(void) { return g_last_error.c_str(); }

int tn_device_info(char *name, uint32_t cap, uint32_t *sm_count) {
  int dev = 0, cnt = 0;
  cudaError_t e = cudaGetDeviceCount(&cnt);
  if (e != cudaSuccess || cnt == 0) {
    g_last_error = "no CUDA device";
    return TN_ERR_NO_DEVICE;
  }
  CK(cudaGetDevice(&dev));
  cudaDeviceProp prop;
  CK(cudaGetDeviceProperties(&prop, dev));
  if (name && cap) {
    std::strncpy(name, prop.name, cap - 1);
    name[cap - 1] = 0;
  }
  if (sm_count) *sm_count = uint32_t(prop.multiProcessorCount);
  return TN_OK;
}

}  // extern "C"

namespace {

int mps_alloc(tn_mps *m) {
  const size_t slot = size_t(2) * m->cap * m->cap * elem_bytes(m->prec);
  CK(m->gamma.ensure(slot * m->n));
  CK(m->lam.ensure(sizeof(double) * size_t(m->cap) * (m->n + 1)));
  CK(m->chi.ensure(sizeof(int) * (m->n + 1)));
  CK(m->status.ensure(sizeof(int)));
  CK(m->dtraj.ensure(sizeof(TrajDev)));
  CK(m->stats.ensure(sizeof(double) * STAT_N));
  CK(cudaMemsetAsync(m->stats.p, 0, sizeof(double) * STAT_N, m->st));
  TrajDev &d = m->h;
  d.stats = m->stats.as<double>();
  d.gamma = m->gamma.p;
  d.lam = m->lam.as<double>();
  d.chi = m->chi.as<int>();
  d.status = m->status.as<int>();
  d.n = int(m->n);
  d.cap = int(m->cap);
  fill_trunc(d, m->has_trunc ? &m->trunc : nullptr);
  CK(cudaMemcpyAsync(m->dtraj.p, &d, sizeof(TrajDev), cudaMemcpyHostToDevice, m->st));
  CK(cudaMemsetAsync(m->status.p, 0, sizeof(int), m->st));
  m->L.ws_cap = int(m->cap);
  {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&m->L.sms, cudaDevAttrMultiProcessorCount, dev);
  }
  m->L.sortP = next_pow2(2 * int(m->cap));
  CK(m->L.ws.ensure(run_work_bytes(m->prec, m->L.ws_cap)));
  return TN_OK;
}

int mps_reset(tn_mps *m) {
  CK(m->L.items.ensure(sizeof(int)));
  int zero = 0;
  CK(cudaMemcpyAsync(m->L.items.p, &zero, sizeof(int), cudaMemcpyHostToDevice, m->st));
  CK(launch_reset(m->dtraj.as<TrajDev>(), m->L.items.as<int>(), 1, m->prec, m->st));
  return TN_OK;
}

// Run one program on the handle.  Outputs are copied back (and the stream
// synchronised) only when a pointer is given.
int mps_run(tn_mps *m, const std::vector<Instr> &prog, const std::vector<double> &gates,
            const std::vector<double> &us, int n_meas_out, int32_t *outc, double *probs, int n_ent_out,
            double *ents, int n_pout, double *pout, const std::vector<Instr> &par = {}) {
  if (prog.empty() && par.empty()) return TN_OK;
  Launcher &L = m->L;
  if (!par.empty()) {
    // independent single-operation items (disjoint gates) spread over SMs
    const int np = int(par.size());
    const int grid = std::max(1, std::min(np, L.sms));
    if (grid > L.ws_ctas) {
      CK(cudaStreamSynchronize(m->st));
      L.ws.release();
      CK(L.ws.ensure(run_work_bytes(m->prec, L.ws_cap) * size_t(grid)));
      L.ws_ctas = grid;
    }
    std::vector<Item> it(np);
    for (int i = 0; i < np; ++i) it[i] = Item{0, i, 1, 0};
    CK(L.gprog.ensure(np * sizeof(Instr)));
    CK(L.gitems.ensure(np * sizeof(Item)));
    CK(L.counter.ensure(2 * sizeof(int)));
    CK(L.gates.ensure(std::max<size_t>(1, gates.size()) * sizeof(double)));
    CK(cudaMemcpyAsync(L.gprog.p, par.data(), np * sizeof(Instr), cudaMemcpyHostToDevice, m->st));
    CK(cudaMemcpyAsync(L.gitems.p, it.data(), np * sizeof(Item), cudaMemcpyHostToDevice, m->st));
    if (!gates.empty())
      CK(cudaMemcpyAsync(L.gates.p, gates.data(), gates.size() * sizeof(double), cudaMemcpyHostToDevice, m->st));
    CK(cudaMemsetAsync(L.counter.p, 0, 2 * sizeof(int), m->st));
    LaunchArgs la{};
    la.items = L.gitems.as<Item>();
    la.nitems = np;
    la.counter = L.counter.as<int>() + 1;
    la.trajs = m->dtraj.as<TrajDev>();
    la.prog = L.gprog.as<Instr>();
    la.gates = L.gates.as<double>();
    la.ws = L.ws.p;
    la.ws_stride = run_work_bytes(m->prec, L.ws_cap);
    la.max_sweeps = kMaxSweeps;
    la.jacobi_scheme = kDefaultScheme;
    CK(launch_run(m->prec, la, grid, L.sortP, L.ws_cap, m->st));
    if (prog.empty()) return TN_OK;
  }
  CK(L.prog.ensure(prog.size() * sizeof(Instr)));
  CK(L.items.ensure(sizeof(Item)));
  CK(L.counter.ensure(sizeof(int)));
  CK(L.gates.ensure(std::max<size_t>(1, gates.size()) * sizeof(double)));
  CK(L.us.ensure(std::max<size_t>(1, us.size()) * sizeof(double)));
  const bool gates_loaded = !par.empty();
  CK(L.outc.ensure(std::max(1, n_meas_out) * sizeof(int)));
  CK(L.probs.ensure(std::max(1, n_meas_out) * sizeof(double)));
  CK(L.ents.ensure(std::max(1, n_ent_out) * sizeof(double)));
  CK(L.pout.ensure(std::max(1, 2 * n_pout) * sizeof(double)));
  CK(cudaMemcpyAsync(L.prog.p, prog.data(), prog.size() * sizeof(Instr), cudaMemcpyHostToDevice, m->st));
  if (!gates.empty() && !gates_loaded)
    CK(cudaMemcpyAsync(L.gates.p, gates.data(), gates.size() * sizeof(double), cudaMemcpyHostToDevice, m->st));
  if (!us.empty())
    CK(cudaMemcpyAsync(L.us.p, us.data(), us.size() * sizeof(double), cudaMemcpyHostToDevice, m->st));
  Item it{0, 0, int(prog.size()), 0};
  CK(cudaMemcpyAsync(L.items.p, &it, sizeof(Item), cudaMemcpyHostToDevice, m->st));
  CK(cudaMemsetAsync(L.counter.p, 0, sizeof(int), m->st));
  LaunchArgs la{};
  la.items = L.items.as<Item>();
  la.nitems = 1;
  la.counter = L.counter.as<int>();
  la.trajs = m->dtraj.as<TrajDev>();
  la.prog = L.prog.as<Instr>();
  la.gates = L.gates.as<double>();
  la.us = L.us.as<double>();
  la.outcomes = L.outc.as<int>();
  la.probs = L.probs.as<double>();
  la.ents = L.ents.as<double>();
  la.pout = L.pout.as<double>();
  la.ws = L.ws.p;
  la.ws_stride = 0;
  la.max_sweeps = kMaxSweeps;
  la.jacobi_scheme = kDefaultScheme;
  CK(launch_run(m->prec, la, 1, L.sortP, L.ws_cap, m->st));
  bool sync = false;
  if (outc && n_meas_out > 0) {
    CK(cudaMemcpyAsync(outc, L.outc.p, n_meas_out * sizeof(int), cudaMemcpyDeviceToHost, m->st));
    sync = true;
  }
  if (probs && n_meas_out > 0) {
    CK(cudaMemcpyAsync(probs, L.probs.p, n_meas_out * sizeof(double), cudaMemcpyDeviceToHost, m->st));
    sync = true;
  }
  if (ents && n_ent_out > 0) {
    CK(cudaMemcpyAsync(ents, L.ents.p, n_ent_out * sizeof(double), cudaMemcpyDeviceToHost, m->st));
    sync = true;
  }
  if (pout && n_pout > 0) {
    CK(cudaMemcpyAsync(pout, L.pout.p, 2 * n_pout * sizeof(double), cudaMemcpyDeviceToHost, m->st));
    sync = true;
  }
  if (sync) CK(cudaStreamSynchronize(m->st));
  return TN_OK;
}

int read_chi(const tn_mps *m, std::vector<int> &chi) {
  chi.resize(m->n + 1);
  CK(cudaMemcpyAsync(chi.data(), m->chi.p, sizeof(int) * (m->n + 1), cudaMemcpyDeviceToHost, m->st));
  CK(cudaStreamSynchronize(m->st));
  return TN_OK;
}

// Gamma of site k as complex128 host values.
int read_gamma(const tn_mps *m, uint32_t k, const std::vector<int> &chi, std::vector<double> &out) {
  const size_t cnt = size_t(chi[k]) * 2 * chi[k + 1];
  out.resize(2 * cnt);
  const size_t slot = size_t(2) * m->cap * m->cap * elem_bytes(m->prec);
  const char *src = reinterpret_cast<const char *>(m->gamma.p) + slot * k;
  if (m->prec == TN_PREC_F64) {
    CK(cudaMemcpyAsync(out.data(), src, cnt * 16, cudaMemcpyDeviceToHost, m->st));
    CK(cudaStreamSynchronize(m->st));
  } else {
    std::vector<char> tmp(cnt * elem_bytes(m->prec));
    CK(cudaMemcpyAsync(tmp.data(), src, tmp.size(), cudaMemcpyDeviceToHost, m->st));
    CK(cudaStreamSynchronize(m->st));
    layout_to_reals(m->prec, tmp.data(), 2 * cnt, out.data());
  }
  return TN_OK;
}

int read_lam(const tn_mps *m, uint32_t b, int len, std::vector<double> &out) {
  out.resize(len);
  CK(cudaMemcpyAsync(out.data(), m->lam.as<double>() + size_t(b + 1) * m->cap, sizeof(double) * len,
                     cudaMemcpyDeviceToHost, m->st));
  CK(cudaStreamSynchronize(m->st));
  return TN_OK;
}

bool gate_shape_ok(uint32_t rows, uint32_t cols, uint32_t d) { return rows == d && cols == d; }

// A non-finite gate entry would spread NaN / inf through the bond's Schmidt
// values and every later operation; it is refused before any device work.
bool all_finite(const double *x, size_t n) {
  for (size_t i = 0; i < n; ++i)
    if (!std::isfinite(x[i])) return false;
  return true;
}

}  // namespace

extern "C" {

int tn_mps_new_qubits(uint32_t n, const tn_trunc *trunc, int32_t precision, uint32_t chi_cap, tn_mps **out) {
  if (!out) return TN_ERR_INVALID_ARG;
  *out = nullptr;
  if (n == 0) return TN_ERR_EMPTY_SYSTEM;
  if (precision != TN_PREC_F64 && precision != TN_PREC_MIXED && precision != TN_PREC_DF) return TN_ERR_INVALID_ARG;
  if (int s = check_trunc(trunc)) return s;
  int cnt = 0;
  if (cudaGetDeviceCount(&cnt) != cudaSuccess || cnt == 0) {
    g_last_error = "no CUDA device";
    return TN_ERR_NO_DEVICE;
  }
  tn_mps *m = new tn_mps();
  m->n = n;
  m->prec = precision;
  m->has_trunc = trunc != nullptr;
  if (trunc) m->trunc = *trunc;
  m->cap = chi_cap ? std::min(chi_cap, max_schmidt_rank(n)) : default_cap(n, trunc);
  if (m->cap < 1) m->cap = 1;
  cudaError_t e = cudaStreamCreateWithFlags(&m->st, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete m;
    return cuda_fail(e, "cudaStreamCreate");
  }
  int s = mps_alloc(m);
  if (s == TN_OK) s = mps_reset(m);
  if (s == TN_OK) {
    e = cudaStreamSynchronize(m->st);
    if (e != cudaSuccess) s = cuda_fail(e, "reset");
  }
  if (s != TN_OK) {
    tn_mps_free(m);
    return s;
  }
  *out = m;
  return TN_OK;
}

int tn_mps_free(tn_mps *m) {
  if (!m) return TN_OK;
  if (m->st) cudaStreamSynchronize(m->st);
  m->gamma.release();
  m->lam.release();
  m->chi.release();
  m->status.release();
  m->dtraj.release();
  m->stats.release();
  m->L.release();
  if (m->st) cudaStreamDestroy(m->st);
  delete m;
  return TN_OK;
}

int tn_mps_clone(const tn_mps *src, tn_mps **out) {
  if (!src || !out) return TN_ERR_INVALID_ARG;
  *out = nullptr;
  tn_mps *m = new tn_mps();
  m->n = src->n;
  m->cap = src->cap;
  m->prec = src->prec;
  m->has_trunc = src->has_trunc;
  m->trunc = src->trunc;
  cudaError_t e = cudaStreamCreateWithFlags(&m->st, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete m;
    return cuda_fail(e, "cudaStreamCreate");
  }
  int s = mps_alloc(m);
  if (s != TN_OK) {
    tn_mps_free(m);
    return s;
  }
  e = cudaStreamSynchronize(src->st);
  const size_t slot = size_t(2) * m->cap * m->cap * elem_bytes(m->prec);
  if (e == cudaSuccess) e = cudaMemcpyAsync(m->gamma.p, src->gamma.p, slot * m->n, cudaMemcpyDeviceToDevice, m->st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(m->lam.p, src->lam.p, sizeof(double) * m->cap * (m->n + 1), cudaMemcpyDeviceToDevice, m->st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(m->chi.p, src->chi.p, sizeof(int) * (m->n + 1), cudaMemcpyDeviceToDevice, m->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(m->st);
  if (e != cudaSuccess) {
    tn_mps_free(m);
    return cuda_fail(e, "clone");
  }
  *out = m;
  return TN_OK;
}

// Checkpoint / resume: a state from its reference-layout parts (the inverse
// of tn_mps_export_gamma + tn_mps_svals).
int tn_mps_import(uint32_t n, const uint32_t *chi, const double *gammas, const double *lams, const tn_trunc *trunc,
                  int32_t precision, uint32_t chi_cap, tn_mps **out) {
  if (!out) return TN_ERR_INVALID_ARG;
  *out = nullptr;
  if (n == 0) return TN_ERR_EMPTY_SYSTEM;
  if (!chi || !gammas || (n > 1 && !lams)) return TN_ERR_INVALID_ARG;
  if (chi[0] != 1 || chi[n] != 1) return TN_ERR_STATE_SHAPE;
  uint32_t widest = 1;
  size_t ng = 0, nl = 0;
  for (uint32_t k = 0; k < n; ++k) {
    if (chi[k + 1] == 0) return TN_ERR_STATE_SHAPE;
    widest = std::max(widest, chi[k + 1]);
    ng += size_t(chi[k]) * 2 * chi[k + 1];
    if (k + 1 < n) nl += chi[k + 1];
  }
  if (!all_finite(gammas, 2 * ng) || (nl && !all_finite(lams, nl))) return TN_ERR_INVALID_ARG;
  uint32_t cap = chi_cap;
  if (!cap) cap = std::max(default_cap(n, trunc), widest);
  if (widest > cap || widest > max_schmidt_rank(n)) return TN_ERR_CAPACITY;
  tn_mps *m = nullptr;
  if (int s = tn_mps_new_qubits(n, trunc, precision, cap, &m)) return s;
  if (m->cap < widest) {
    tn_mps_free(m);
    return TN_ERR_CAPACITY;
  }
  const size_t slot = size_t(2) * m->cap * m->cap * elem_bytes(m->prec);
  std::vector<int> ichi(chi, chi + n + 1);
  std::vector<char> tmp;
  cudaError_t e = cudaStreamSynchronize(m->st);
  size_t go = 0, lo = 0;
  for (uint32_t k = 0; k < n && e == cudaSuccess; ++k) {
    const size_t cnt = size_t(chi[k]) * 2 * chi[k + 1];  // complex entries of Gamma_k
    char *dst = static_cast<char *>(m->gamma.p) + slot * k;
    if (m->prec == TN_PREC_F64) {
      e = cudaMemcpy(dst, gammas + 2 * go, cnt * 16, cudaMemcpyHostToDevice);
    } else {
      tmp.resize(cnt * elem_bytes(m->prec));
      reals_to_layout(m->prec, gammas + 2 * go, 2 * cnt, tmp.data());
      e = cudaMemcpy(dst, tmp.data(), tmp.size(), cudaMemcpyHostToDevice);
    }
    go += cnt;
    if (e == cudaSuccess && k + 1 < n) {
      e = cudaMemcpy(m->lam.as<double>() + size_t(k + 1) * m->cap, lams + lo, sizeof(double) * chi[k + 1],
                     cudaMemcpyHostToDevice);
      lo += chi[k + 1];
    }
  }
  if (e == cudaSuccess) e = cudaMemcpy(m->chi.p, ichi.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    tn_mps_free(m);
    return cuda_fail(e, "import");
  }
  *out = m;
  return TN_OK;
}

int tn_mps_n(const tn_mps *m, uint32_t *n) {
  if (!m || !n) return TN_ERR_INVALID_ARG;
  *n = m->n;
  return TN_OK;
}

int tn_mps_precision(const tn_mps *m, int32_t *precision) {
  if (!m || !precision) return TN_ERR_INVALID_ARG;
  *precision = m->prec;
  return TN_OK;
}

int tn_mps_get_trunc(const tn_mps *m, tn_trunc *out) {
  if (!m || !out) return TN_ERR_INVALID_ARG;
  if (!m->has_trunc) return TN_NONE;
  *out = m->trunc;
  return TN_OK;
}

int tn_mps_set_trunc(tn_mps *m, const tn_trunc *trunc) {
  if (!m) return TN_ERR_INVALID_ARG;
  if (int s = check_trunc(trunc)) return s;
  m->has_trunc = trunc != nullptr;
  if (trunc) m->trunc = *trunc;
  fill_trunc(m->h, trunc);
  CK(cudaMemcpyAsync(m->dtraj.p, &m->h, sizeof(TrajDev), cudaMemcpyHostToDevice, m->st));
  CK(cudaStreamSynchronize(m->st));
  return TN_OK;
}

int tn_mps_apply_unitary1(tn_mps *m, uint32_t k, const double *op, uint32_t rows, uint32_t cols) {
  if (!m || !op) return TN_ERR_INVALID_ARG;
  if (k >= m->n) return TN_OK;
  if (!gate_shape_ok(rows, cols, 2)) return TN_ERR_OPERATOR_SHAPE;
  if (!all_finite(op, 8)) return TN_ERR_INVALID_ARG;
  std::vector<double> g(32, 0.0);
  std::memcpy(g.data(), op, 8 * sizeof(double));
  return mps_run(m, {Instr{OP_UNI1, int(k), 0, 0}}, g, {}, 0, nullptr, nullptr, 0, nullptr, 0, nullptr);
}

int tn_mps_apply_unitary2(tn_mps *m, uint32_t k, const double *op, uint32_t rows, uint32_t cols) {
  if (!m || !op) return TN_ERR_INVALID_ARG;
  if (m->n == 1 || k >= m->n - 1) return TN_OK;
  if (!gate_shape_ok(rows, cols, 4)) return TN_ERR_OPERATOR_SHAPE;
  if (!all_finite(op, 32)) return TN_ERR_INVALID_ARG;
  std::vector<double> g(op, op + 32);
  return mps_run(m, {Instr{OP_GATE, int(k), 0, 0}}, g, {}, 0, nullptr, nullptr, 0, nullptr, 0, nullptr);
}

int tn_mps_probs(const tn_mps *cm, uint32_t k, double out[2]) {
  tn_mps *m = const_cast<tn_mps *>(cm);
  if (!m || !out) return TN_ERR_INVALID_ARG;
  if (k >= m->n) return TN_NONE;
  return mps_run(m, {Instr{OP_PROBS, int(k), 0, 0}}, {}, {}, 0, nullptr, nullptr, 0, nullptr, 1, out);
}

int tn_mps_prob(const tn_mps *m, uint32_t k, uint32_t p, double *out) {
  if (!m || !out) return TN_ERR_INVALID_ARG;
  if (k >= m->n || p >= 2) return TN_NONE;
  double pr[2];
  int s = tn_mps_probs(m, k, pr);
  if (s == TN_OK) *out = pr[p];
  return s;
}

int tn_mps_measure_prob(tn_mps *m, uint32_t k, double u, int32_t *outcome, double *prob) {
  if (!m) return TN_ERR_INVALID_ARG;
  if (k >= m->n) return TN_NONE;
  if (!std::isfinite(u)) return TN_ERR_INVALID_ARG;
  std::vector<Instr> prog{Instr{OP_MEAS, int(k), 0, -1}};
  emit_sweep(prog, m->n);
  int32_t oc = 0;
  double pr = 0.0;
  int s = mps_run(m, prog, {}, {u}, 1, &oc, &pr, 0, nullptr, 0, nullptr);
  if (s != TN_OK) return s;
  if (outcome) *outcome = oc;
  if (prob) *prob = pr;
  return TN_OK;
}

int tn_mps_measure_postsel_prob(tn_mps *m, uint32_t k, uint32_t p, double *prob) {
  if (!m) return TN_ERR_INVALID_ARG;
  if (k >= m->n || p >= 2) return TN_NONE;
  std::vector<Instr> prog{Instr{OP_MEAS, int(k), 0, int(p)}};
  emit_sweep(prog, m->n);
  int32_t oc = 0;
  double pr = 0.0;
  int s = mps_run(m, prog, {}, {0.0}, 1, &oc, &pr, 0, nullptr, 0, nullptr);
  if (s == TN_OK && prob) *prob = pr;
  return s;
}

}  // extern "C"

namespace {

// filter k < n, stable sort by k, keep first of each k (mps.rs:2212-2219)
void select_targets(uint32_t n, const uint32_t *ks, uint32_t nk, const int32_t *posts, std::vector<uint32_t> &tk,
                    std::vector<int32_t> &tp) {
  std::vector<std::pair<uint32_t, uint32_t>> v;
  for (uint32_t i = 0; i < nk; ++i)
    if (ks[i] < n) v.push_back({ks[i], i});
  std::stable_sort(v.begin(), v.end(), [](auto &a, auto &b) { return a.first < b.first; });
  tk.clear();
  tp.clear();
  for (size_t i = 0; i < v.size(); ++i) {
    if (i > 0 && v[i].first == v[i - 1].first) continue;
    tk.push_back(v[i].first);
    if (posts) tp.push_back(posts[v[i].second]);
  }
}

}  // namespace

extern "C" {

int tn_mps_apply_meas_prob_layer(tn_mps *m, const uint32_t *ks, uint32_t nk, const int32_t *posts, const double *us,
                                 uint32_t *out_ks, int32_t *outcomes, double *probs, uint32_t *n_out) {
  if (!m || (nk && !ks)) return TN_ERR_INVALID_ARG;
  std::vector<uint32_t> tk;
  std::vector<int32_t> tp;
  select_targets(m->n, ks, nk, posts, tk, tp);
  if (n_out) *n_out = uint32_t(tk.size());
  if (tk.empty()) return TN_OK;
  for (auto &p : tp)
    if (p > 1) p = 1;  // invalid quantum numbers are the caller's error; clamp
  if (!us && tp.empty()) return TN_ERR_INVALID_ARG;
  std::vector<double> u(tk.size(), 0.0);
  if (us)
    for (size_t j = 0; j < tk.size(); ++j) u[j] = us[j];
  if (!all_finite(u.data(), u.size())) return TN_ERR_INVALID_ARG;
  std::vector<Instr> prog;
  emit_meas_layer(prog, m->n, tk, tp, 0);
  std::vector<int32_t> oc(tk.size());
  std::vector<double> pr(tk.size());
  int s = mps_run(m, prog, {}, u, int(tk.size()), oc.data(), pr.data(), 0, nullptr, 0, nullptr);
  if (s != TN_OK) return s;
  for (size_t j = 0; j < tk.size(); ++j) {
    if (out_ks) out_ks[j] = tk[j];
    if (outcomes) outcomes[j] = oc[j];
    if (probs) probs[j] = pr[j];
  }
  return TN_OK;
}

int tn_mps_apply_bilayer(tn_mps *m, const uint32_t *gate_ks, const double *gates, uint32_t ng,
                         const uint32_t *meas_ks, uint32_t nm, const double *us, uint32_t *out_ks,
                         int32_t *outcomes, double *probs, uint32_t *n_out) {
  if (!m || (ng && (!gate_ks || !gates)) || (nm && (!meas_ks || !us))) return TN_ERR_INVALID_ARG;
  if (ng && !all_finite(gates, size_t(ng) * 32)) return TN_ERR_INVALID_ARG;
  std::vector<Instr> prog, par;
  std::vector<double> g;
  g.reserve(size_t(ng) * 32);
  bool disjoint = true;
  for (uint32_t i = 0; i < ng && disjoint; ++i)
    for (uint32_t j = i + 1; j < ng; ++j)
      if ((gate_ks[i] > gate_ks[j] ? gate_ks[i] - gate_ks[j] : gate_ks[j] - gate_ks[i]) < 2) {
        disjoint = false;
        break;
      }
  for (uint32_t i = 0; i < ng; ++i) {
    if (m->n == 1 || gate_ks[i] >= m->n - 1) continue;
    (disjoint ? par : prog).push_back(Instr{OP_GATE, int(gate_ks[i]), int(g.size() / 32), 0});
    g.insert(g.end(), gates + size_t(i) * 32, gates + size_t(i + 1) * 32);
  }
  std::vector<uint32_t> tk;
  std::vector<int32_t> tp;
  select_targets(m->n, meas_ks, nm, nullptr, tk, tp);
  std::vector<double> u(us, us + tk.size());
  if (!all_finite(u.data(), u.size())) return TN_ERR_INVALID_ARG;
  emit_meas_layer(prog, m->n, tk, tp, 0);
  if (n_out) *n_out = uint32_t(tk.size());
  std::vector<int32_t> oc(std::max<size_t>(1, tk.size()));
  std::vector<double> pr(std::max<size_t>(1, tk.size()));
  int s = mps_run(m, prog, g, u, int(tk.size()), tk.empty() ? nullptr : oc.data(), tk.empty() ? nullptr : pr.data(),
                  0, nullptr, 0, nullptr, par);
  if (s != TN_OK) return s;
  for (size_t j = 0; j < tk.size(); ++j) {
    if (out_ks) out_ks[j] = tk[j];
    if (outcomes) outcomes[j] = oc[j];
    if (probs) probs[j] = pr[j];
  }
  return TN_OK;
}

int tn_mps_entropy_vn(const tn_mps *cm, uint32_t b, double *out) {
  tn_mps *m = const_cast<tn_mps *>(cm);
  if (!m || !out) return TN_ERR_INVALID_ARG;
  if (m->n < 2 || b >= m->n - 1) return TN_NONE;
  return mps_run(m, {Instr{OP_ENTROPY, int(b), 0, 0}}, {}, {}, 0, nullptr, nullptr, 1, out, 0, nullptr);
}

int tn_mps_entropy_ry_schmidt(const tn_mps *cm, double a, uint32_t b, double *out) {
  tn_mps *m = const_cast<tn_mps *>(cm);
  if (!m || !out) return TN_ERR_INVALID_ARG;
  if (a == 1.0) return tn_mps_entropy_vn(cm, b, out);
  if (m->n < 2 || b >= m->n - 1) return TN_NONE;
  return mps_run(m, {Instr{OP_RENYI, int(b), 0, 0}}, {}, {a}, 0, nullptr, nullptr, 1, out, 0, nullptr);
}

int tn_mps_bond_dim(const tn_mps *m, uint32_t b, uint32_t *out) {
  if (!m || !out) return TN_ERR_INVALID_ARG;
  if (m->n < 2 || b >= m->n - 1) return TN_NONE;
  std::vector<int> chi;
  if (int s = read_chi(m, chi)) return s;
  *out = uint32_t(chi[b + 1]);
  return TN_OK;
}

int tn_mps_max_bond_dim(const tn_mps *m, uint32_t *out) {
  if (!m || !out) return TN_ERR_INVALID_ARG;
  if (m->n < 2) return TN_NONE;
  std::vector<int> chi;
  if (int s = read_chi(m, chi)) return s;
  *out = uint32_t(*std::max_element(chi.begin() + 1, chi.end() - 1));
  return TN_OK;
}

int tn_mps_svals(const tn_mps *m, uint32_t b, double *out, uint32_t cap, uint32_t *len) {
  if (!m) return TN_ERR_INVALID_ARG;
  if (m->n < 2 || b >= m->n - 1) return TN_NONE;
  std::vector<int> chi;
  if (int s = read_chi(m, chi)) return s;
  const int l = chi[b + 1];
  if (len) *len = uint32_t(l);
  if (!out) return TN_OK;
  if (cap < uint32_t(l)) return TN_ERR_INVALID_ARG;
  std::vector<double> v;
  if (int s = read_lam(m, b, l, v)) return s;
  std::memcpy(out, v.data(), sizeof(double) * l);
  return TN_OK;
}

int tn_mps_export_gamma(const tn_mps *m, uint32_t k, double *out, uint64_t cap, uint32_t dims[3]) {
  if (!m) return TN_ERR_INVALID_ARG;
  if (k >= m->n) return TN_NONE;
  std::vector<int> chi;
  if (int s = read_chi(m, chi)) return s;
  if (dims) {
    dims[0] = uint32_t(chi[k]);
    dims[1] = 2;
    dims[2] = uint32_t(chi[k + 1]);
  }
  if (!out) return TN_OK;
  const uint64_t need = uint64_t(chi[k]) * 2 * chi[k + 1] * 2;
  if (cap < need) return TN_ERR_INVALID_ARG;
  std::vector<double> g;
  if (int s = read_gamma(m, k, chi, g)) return s;
  std::memcpy(out, g.data(), sizeof(double) * need);
  return TN_OK;
}

// contract (mps.rs:794-798): psi <- (psi * Lambda_{k-1}) . Gamma_k, on the host.
int tn_mps_contract(const tn_mps *m, double *out, uint64_t cap) {
  if (!m || !out) return TN_ERR_INVALID_ARG;
  if (m->n > 24) return TN_ERR_INVALID_ARG;
  const uint64_t dim = uint64_t(1) << m->n;
  if (cap < 2 * dim) return TN_ERR_INVALID_ARG;
  std::vector<int> chi;
  if (int s = read_chi(m, chi)) return s;
  std::vector<double> psi;  // (rows, chi) complex, rows = 2^k
  if (int s = read_gamma(m, 0, chi, psi)) return s;
  uint64_t rows = 2;
  for (uint32_t k = 1; k < m->n; ++k) {
    const int cl = chi[k], cr = chi[k + 1];
    std::vector<double> lam, g;
    if (int s = read_lam(m, k - 1, cl, lam)) return s;
    if (int s = read_gamma(m, k, chi, g)) return s;
    std::vector<double> nxt(2 * rows * 2 * cr, 0.0);
    for (uint64_t r = 0; r < rows; ++r)
      for (int v = 0; v < cl; ++v) {
        const double pr = psi[2 * (r * cl + v)] * lam[v], pi = psi[2 * (r * cl + v) + 1] * lam[v];
        if (pr == 0.0 && pi == 0.0) continue;
        for (int s = 0; s < 2; ++s)
          for (int w = 0; w < cr; ++w) {
            const size_t gi = 2 * ((size_t(v) * 2 + s) * cr + w);
            const size_t oi = 2 * (((r * 2 + s) * cr) + w);
            nxt[oi] += pr * g[gi] - pi * g[gi + 1];
            nxt[oi + 1] += pr * g[gi + 1] + pi * g[gi];
          }
      }
    psi.swap(nxt);
    rows *= 2;
  }
  std::memcpy(out, psi.data(), sizeof(double) * 2 * dim);
  return TN_OK;
}

}  // extern "C"

int tn::mps_view(const tn_mps *m, tn::MpsView *out) {
  if (!m || !out) return TN_ERR_INVALID_ARG;
  out->dtraj = m->dtraj.as<TrajDev>();
  out->n = int(m->n);
  out->cap = int(m->cap);
  out->prec = m->prec;
  out->st = m->st;
  return TN_OK;
}

extern "C" {

int tn_mps_stats(tn_mps *m, double *out, int32_t reset) {
  if (!m) return TN_ERR_INVALID_ARG;
  if (out) CK(cudaMemcpyAsync(out, m->stats.p, sizeof(double) * STAT_N, cudaMemcpyDeviceToHost, m->st));
  if (reset) CK(cudaMemsetAsync(m->stats.p, 0, sizeof(double) * STAT_N, m->st));
  CK(cudaStreamSynchronize(m->st));
  return TN_OK;
}

int tn_mps_device_status(tn_mps *m, int32_t *status) {
  if (!m || !status) return TN_ERR_INVALID_ARG;
  int v = 0;
  CK(cudaMemcpyAsync(&v, m->status.p, sizeof(int), cudaMemcpyDeviceToHost, m->st));
  CK(cudaMemsetAsync(m->status.p, 0, sizeof(int), m->st));
  CK(cudaStreamSynchronize(m->st));
  *status = v;
  return TN_OK;
}

}  // extern "C"
