// tn_batch.cpp -- batch of independent trajectories advanced one brickwork
// layer per persistent launch (the reference runs trajectories one per rayon
// thread, workspace/src/haar_coev_probs.rs:164; here they share one launch).
//
// Per step:  H2D of the packed layer inputs (one copy from pinned memory)
//            -> k_compile (instruction lists on the device)
//            -> k_run (persistent CTAs pull trajectories, most expensive first)
//            -> D2H of outcomes / probabilities / entropies (one copy).
// The device-input variant skips both copies and replays a captured CUDA
// graph of compile + run.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <numeric>
#include <string>
#include <vector>

#include "tn_internal.h"
#include "tn_mps.h"

using namespace tn;

extern "C" const char *tn_last_error(void);

namespace {

int fail(cudaError_t e, const char *what) {
  tn::set_last_error(what, e);
  if (e == cudaErrorMemoryAllocation) return TN_ERR_OOM;
  return TN_ERR_CUDA;
}

#define CKB(call)                                   \
  do {                                              \
    cudaError_t e__ = (call);                       \
    if (e__ != cudaSuccess) return fail(e__, #call); \
  } while (0)

uint32_t max_rank(uint32_t n) { return n / 2 >= 20 ? (1u << 20) : (1u << (n / 2)); }

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

constexpr int kCounters = 16;

}  // namespace

struct tn_batch {
  int prec = TN_PREC_MIXED;
  uint32_t ntraj = 0;
  cudaStream_t st = nullptr;
  int sms = 1, bps = 1, grid_max = 1;
  int maxcap = 1, maxn = 1, sortP = 1, pcap = 8;
  int scheme = kDefaultScheme, max_sweeps = 40;  // Jacobi tuning (tn_batch_set_tuning)
  int theta_simt = 0;               // 1: SIMT theta contraction instead of the tensor-core one
  // Online autotuner (tn_batch_autotune): the next steps run each candidate
  // configuration for `trial` steps; the score of a candidate is launch time
  // per algorithmic flop (both measured on the device); the best one stays.
  struct Tuner {
    bool on = false, pending = false;
    int trial = 1, cand = 0, in_cand = 0;
    double flops0 = 0;
    std::vector<double> score;
  } tune;
  std::vector<uint32_t> n_alloc, cap;
  std::vector<TrajDev> h;
  std::vector<size_t> slot_bytes;
  void *arena = nullptr;
  TrajDev *dtraj = nullptr;
  int *dstatus = nullptr;
  double *dstats = nullptr;
  void *ws = nullptr;
  size_t ws_stride = 0;
  // step buffers: one packed device block + one pinned host block
  void *dstep = nullptr, *hstep = nullptr;
  size_t step_bytes = 0;
  uint32_t step_nt = 0, step_ng = 0, step_nm = 0;
  Instr *dprog = nullptr;
  Item *ditems = nullptr;
  Instr *dgprog = nullptr;  // one single-gate program per gate of the layer
  Item *dgitems = nullptr;
  int gcap = 0;
  uint32_t sum_n = 0;
  // [0] queue head, [1] reset list, [2] second-launch queue, [3] gate count, [4..8) bind staging,
  // [8] push counter, [9] queue-wait error, [10] sweep head
  int *dcounter = nullptr;
  int schedule = 1;  // 1: one launch per layer, sweeps pushed as gates finish; 0: two launches
  int *drem = nullptr, *dgstart = nullptr, *dscratch = nullptr, *dorder = nullptr;
  Item *ddyn = nullptr;
  // device-input mode
  void *din = nullptr;
  uint32_t din_gates = 0, din_meas = 0;
  std::map<uint32_t, cudaGraphExec_t> graphs;
  cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};  // around the gate and sweep launches
  bool ev_recorded = false;
  bool ev_one_launch = false;  // the recorded step ran the one-launch schedule
  cudaEvent_t ev_done = nullptr;  // end of the last host-input step (outputs in pinned memory)
  // device interval of the last host-input step between its input copy and
  // its output copy (every kernel of the step, inputs resident in HBM)
  cudaEvent_t ev_step[2] = {nullptr, nullptr};
  // limit of a CTA's wait for a pushed sweep item (0: kQueueWaitNs), and
  // sweep slots that no item ever fills (a test of that limit)
  unsigned long long queue_wait_ns = 0;
  uint32_t phantom_sweeps = 0;
  bool ev_step_recorded = false;
  uint32_t pending_nt = 0, pending_nm = 0;
  bool async_step = false;        // engine mode: tn_batch_step returns before the outputs arrive
  int grid_limit = 0;             // engine mode: CTAs per launch (0 = every resident CTA)
};

namespace {

// Packed per-step layout (same offsets on host and device).
struct StepLayout {
  size_t list, order, goff, gks, moff, mks, posts, gates, us, outc, probs, ents, total, in_bytes, out_off;
};

StepLayout step_layout(uint32_t nt, uint32_t ng, uint32_t nm) {
  StepLayout L{};
  size_t p = 0;
  auto take = [&](size_t bytes) {
    size_t o = p;
    p = align256(p + bytes);
    return o;
  };
  L.gates = take(sizeof(double) * 32 * std::max<uint32_t>(ng, 1));
  L.us = take(sizeof(double) * std::max<uint32_t>(nm, 1));
  L.list = take(sizeof(int) * std::max<uint32_t>(nt, 1));
  L.order = take(sizeof(int) * std::max<uint32_t>(nt, 1));
  L.goff = take(sizeof(int) * (nt + 1));
  L.gks = take(sizeof(int) * std::max<uint32_t>(ng, 1));
  L.moff = take(sizeof(int) * (nt + 1));
  L.mks = take(sizeof(int) * std::max<uint32_t>(nm, 1));
  L.posts = take(sizeof(int) * std::max<uint32_t>(nm, 1));
  L.in_bytes = p;
  L.out_off = p;
  L.outc = take(sizeof(int) * std::max<uint32_t>(nm, 1));
  L.probs = take(sizeof(double) * std::max<uint32_t>(nm, 1));
  L.ents = take(sizeof(double) * std::max<uint32_t>(nt, 1));
  L.total = p;
  return L;
}

int ensure_step(tn_batch *b, uint32_t nt, uint32_t ng, uint32_t nm) {
  if (nt <= b->step_nt && ng <= b->step_ng && nm <= b->step_nm && b->dstep) return TN_OK;
  for (auto &kv : b->graphs) cudaGraphExecDestroy(kv.second);  // they point at the old buffers
  b->graphs.clear();
  uint32_t NT = std::max(nt, b->step_nt), NG = std::max(ng, b->step_ng), NM = std::max(nm, b->step_nm);
  StepLayout L = step_layout(NT, NG, NM);
  if (b->dstep) cudaFree(b->dstep);
  if (b->hstep) cudaFreeHost(b->hstep);
  if (b->dprog) cudaFree(b->dprog);
  b->dstep = b->hstep = nullptr;
  b->dprog = nullptr;
  CKB(cudaMalloc(&b->dstep, L.total));
  CKB(cudaMallocHost(&b->hstep, L.total));
  b->gcap = int(std::max<uint32_t>(NG, b->sum_n));
  const size_t pbytes = sizeof(Instr) * size_t(NT) * b->pcap, ibytes = sizeof(Item) * NT;
  const size_t gpbytes = sizeof(Instr) * size_t(b->gcap), gibytes = sizeof(Item) * size_t(b->gcap);
  const size_t nbytes = sizeof(int) * NT;
  CKB(cudaMalloc(reinterpret_cast<void **>(&b->dprog),
                 align256(pbytes) + 2 * align256(ibytes) + align256(gpbytes) + align256(gibytes) +
                     4 * align256(nbytes) + 256));
  char *base = reinterpret_cast<char *>(b->dprog);
  size_t at = align256(pbytes);
  auto take = [&](size_t bytes) {
    char *q = base + at;
    at += align256(bytes);
    return q;
  };
  b->ditems = reinterpret_cast<Item *>(take(ibytes));
  b->dgprog = reinterpret_cast<Instr *>(take(gpbytes));
  b->dgitems = reinterpret_cast<Item *>(take(gibytes));
  b->ddyn = reinterpret_cast<Item *>(take(ibytes));
  b->drem = reinterpret_cast<int *>(take(nbytes));
  b->dgstart = reinterpret_cast<int *>(take(nbytes));
  b->dscratch = reinterpret_cast<int *>(take(nbytes));
  b->dorder = reinterpret_cast<int *>(take(nbytes));
  b->step_nt = NT;
  b->step_ng = NG;
  b->step_nm = NM;
  b->step_bytes = L.total;
  return TN_OK;
}

struct StepPtrs {
  const int *list, *order, *goff, *gks, *moff, *mks;
  const int *posts = nullptr;  // per measurement: 0 / 1 post-selected (Meas::Proj), else sampled; null = all sampled
  const double *gates, *us;
  int *outc;
  double *probs, *ents;
};

StepPtrs ptrs_of(const StepLayout &L, char *dbase) {
  StepPtrs p;
  p.list = reinterpret_cast<const int *>(dbase + L.list);
  p.order = reinterpret_cast<const int *>(dbase + L.order);
  p.goff = reinterpret_cast<const int *>(dbase + L.goff);
  p.gks = reinterpret_cast<const int *>(dbase + L.gks);
  p.moff = reinterpret_cast<const int *>(dbase + L.moff);
  p.mks = reinterpret_cast<const int *>(dbase + L.mks);
  p.gates = reinterpret_cast<const double *>(dbase + L.gates);
  p.us = reinterpret_cast<const double *>(dbase + L.us);
  p.outc = reinterpret_cast<int *>(dbase + L.outc);
  p.probs = reinterpret_cast<double *>(dbase + L.probs);
  p.ents = reinterpret_cast<double *>(dbase + L.ents);
  return p;
}

// Candidate configurations of the autotuner: {schedule, Jacobi scheme, SIMT theta}.
constexpr int kTuneCands = 4;
constexpr int kTuneTable[kTuneCands][3] = {{1, 3, 0}, {1, 0, 0}, {0, 3, 0}, {1, 3, 1}};

// Algorithmic flops counted so far over every slot (theta + SVD counters).
int stats_flops(tn_batch *b, double *flops) {
  std::vector<double> v(size_t(STAT_N) * b->ntraj);
  CKB(cudaMemcpyAsync(v.data(), b->dstats, sizeof(double) * v.size(), cudaMemcpyDeviceToHost, b->st));
  CKB(cudaStreamSynchronize(b->st));
  double f = 0.0;
  for (uint32_t t = 0; t < b->ntraj; ++t) f += v[size_t(t) * STAT_N + STAT_FLOP_THETA] + v[size_t(t) * STAT_N + STAT_FLOP_SVD];
  *flops = f;
  return TN_OK;
}

void apply_cfg(tn_batch *b, int c) {
  b->schedule = kTuneTable[c][0];
  b->scheme = kTuneTable[c][1];
  b->theta_simt = kTuneTable[c][2];
}

// Before a host-launched step: score the previous trial step, move on, and
// apply the configuration of this step.
int tune_before(tn_batch *b) {
  tn_batch::Tuner &T = b->tune;
  if (!T.on) return TN_OK;
  if (T.pending) {
    CKB(cudaEventSynchronize(b->ev[2]));
    float g = 0.f, w = 0.f;
    CKB(cudaEventElapsedTime(&g, b->ev[0], b->ev[1]));
    if (!b->ev_one_launch) CKB(cudaEventElapsedTime(&w, b->ev[1], b->ev[2]));
    double f1 = 0.0;
    if (int s = stats_flops(b, &f1)) return s;
    const double df = f1 - T.flops0;
    T.score[T.cand] += df > 0 ? 1e-3 * (g + w) / df : 0.0;
    T.pending = false;
    if (++T.in_cand >= T.trial) {
      T.in_cand = 0;
      if (++T.cand >= kTuneCands) {  // done: keep the best
        int best = 0;
        for (int c = 1; c < kTuneCands; ++c)
          if (T.score[c] < T.score[best]) best = c;
        apply_cfg(b, best);
        T.on = false;
        for (auto &kv : b->graphs) cudaGraphExecDestroy(kv.second);
        b->graphs.clear();
        return TN_OK;
      }
    }
  }
  apply_cfg(b, T.cand);
  return stats_flops(b, &T.flops0);
}

int launch_step(tn_batch *b, uint32_t nt, const StepPtrs &P0, bool timed = true) {
  StepPtrs P = P0;
  if (!P.order) {  // most expensive trajectories first, by their current bond dimensions
    CKB(launch_lpt_order(b->dtraj, P.list, int(nt), P.moff, b->dorder, b->st));
    P.order = b->dorder;
  }
  LaunchArgs la{};
  la.trajs = b->dtraj;
  la.gates = P.gates;
  la.us = P.us;
  la.outcomes = P.outc;
  la.probs = P.probs;
  la.ents = P.ents;
  la.pout = P.probs;
  la.ws = b->ws;
  la.ws_stride = b->ws_stride;
  la.max_sweeps = b->max_sweeps;
  la.jacobi_scheme = b->scheme;
  la.theta_simt = b->theta_simt;
  la.qerr = b->dcounter + 9;
  const int gmax = b->grid_limit > 0 ? std::min(b->grid_limit, b->grid_max) : b->grid_max;
  if (b->schedule == 1) {
    // One launch: gate items (most expensive trajectories first), then each
    // trajectory's sweep program as soon as its last gate item has finished.
    CKB(cudaMemsetAsync(b->dcounter, 0, 4 * sizeof(int), b->st));
    CKB(cudaMemsetAsync(b->dcounter + 8, 0, 3 * sizeof(int), b->st));  // push tail, queue error, sweep head
    const uint32_t phantom = std::min<uint32_t>(b->phantom_sweeps, b->step_nt - std::min(b->step_nt, nt));
    CKB(cudaMemsetAsync(b->ddyn, 0, sizeof(Item) * (nt + phantom), b->st));
    CKB(launch_compile_dd(b->dtraj, P.list, int(nt), P.order, P.goff, P.gks, P.moff, P.mks, P.posts, b->pcap,
                          b->dprog, b->ditems, b->dgprog, b->dgitems, b->gcap, b->dcounter + 3, b->dgstart,
                          b->dscratch, b->drem, b->ddyn, b->dcounter + 8, b->st));
    la.counter = b->dcounter;
    la.items = b->dgitems;
    la.nitems = 0;
    la.nitems_dev = b->dcounter + 3;
    la.prog = b->dprog;
    la.gprog = b->dgprog;
    la.rem = b->drem;
    la.sweeps = b->ditems;
    la.dyn = b->ddyn;
    la.dyn_tail = b->dcounter + 8;
    la.dyn_head = b->dcounter + 10;
    la.nsweeps = int(nt + phantom);
    la.queue_wait_ns = b->queue_wait_ns;
    if (timed) CKB(cudaEventRecord(b->ev[0], b->st));
    CKB(launch_run(b->prec, la, gmax, b->sortP, b->maxcap, b->st));
    if (timed) {
      CKB(cudaEventRecord(b->ev[1], b->st));
      CKB(cudaEventRecord(b->ev[2], b->st));
      b->ev_recorded = true;
      b->ev_one_launch = true;
      b->tune.pending = b->tune.on;
    }
    return TN_OK;
  }
  CKB(launch_compile(b->dtraj, P.list, int(nt), P.order, P.goff, P.gks, P.moff, P.mks, P.posts, b->pcap, b->dprog,
                     b->ditems, b->dgprog, b->dgitems, b->gcap, b->dcounter + 3, b->st));
  CKB(cudaMemsetAsync(b->dcounter, 0, 3 * sizeof(int), b->st));
  la.counter = b->dcounter;
  // launch 1: every gate of the layer is an independent item
  la.items = b->dgitems;
  la.prog = b->dgprog;
  la.nitems = 0;
  la.nitems_dev = b->dcounter + 3;
  if (timed) CKB(cudaEventRecord(b->ev[0], b->st));
  CKB(launch_run(b->prec, la, gmax, b->sortP, b->maxcap, b->st));
  if (timed) CKB(cudaEventRecord(b->ev[1], b->st));
  // launch 2: one measurement-layer program per trajectory
  la.items = b->ditems;
  la.prog = b->dprog;
  la.nitems = int(nt);
  la.nitems_dev = nullptr;
  la.counter = b->dcounter + 2;
  const int grid = std::min<int>(int(nt), gmax);
  CKB(launch_run(b->prec, la, grid, b->sortP, b->maxcap, b->st));
  if (timed) {
    CKB(cudaEventRecord(b->ev[2], b->st));
    b->ev_recorded = true;
    b->ev_one_launch = false;
    b->tune.pending = b->tune.on;
  }
  return TN_OK;
}

}  // namespace

extern "C" {

int tn_batch_create(uint32_t ntraj, const uint32_t *ns, const tn_trunc *truncs, int32_t precision,
                    const uint32_t *chi_caps, tn_batch **out) {
  if (!out || !ns || ntraj == 0) return TN_ERR_INVALID_ARG;
  *out = nullptr;
  if (precision != TN_PREC_F64 && precision != TN_PREC_MIXED && precision != TN_PREC_DF) return TN_ERR_INVALID_ARG;
  for (uint32_t i = 0; i < ntraj; ++i) {
    if (ns[i] == 0) return TN_ERR_EMPTY_SYSTEM;
    if (truncs && (truncs[i].mode < 0 || truncs[i].mode > 3)) return TN_ERR_INVALID_ARG;
  }
  int cnt = 0;
  if (cudaGetDeviceCount(&cnt) != cudaSuccess || cnt == 0) return TN_ERR_NO_DEVICE;
  tn_batch *b = new tn_batch();
  b->prec = precision;
  b->ntraj = ntraj;
  b->n_alloc.assign(ns, ns + ntraj);
  b->cap.resize(ntraj);
  b->h.resize(ntraj);
  b->slot_bytes.resize(ntraj);
  const size_t eb = prec_elem_bytes(precision);
  std::vector<size_t> off(ntraj);
  size_t total = 0;
  for (uint32_t i = 0; i < ntraj; ++i) {
    uint32_t c;
    if (chi_caps && chi_caps[i])
      c = std::min(chi_caps[i], max_rank(ns[i]));
    else if (truncs && (truncs[i].mode == TN_TRUNC_CONST || truncs[i].mode == TN_TRUNC_BOTH))
      c = std::min(std::max<uint32_t>(1, truncs[i].chi_max), max_rank(ns[i]));
    else
      c = std::min<uint32_t>(max_rank(ns[i]), 256);
    b->cap[i] = c;
    size_t bytes = align256(size_t(2) * c * c * eb * ns[i]) + align256(sizeof(double) * size_t(c) * (ns[i] + 1)) +
                   align256(sizeof(int) * (ns[i] + 1));
    off[i] = total;
    b->slot_bytes[i] = bytes;
    total += bytes;
    b->maxcap = std::max<int>(b->maxcap, int(c));
    b->maxn = std::max<int>(b->maxn, int(ns[i]));
    b->sum_n += ns[i];
  }
  auto bail = [&](int s) {
    tn_batch_free(b);
    return s;
  };
  cudaError_t e = cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking);
  if (e != cudaSuccess) return bail(fail(e, "cudaStreamCreate"));
  for (auto &ev : b->ev) {
    e = cudaEventCreate(&ev);
    if (e != cudaSuccess) return bail(fail(e, "cudaEventCreate"));
  }
  e = cudaEventCreateWithFlags(&b->ev_done, cudaEventDisableTiming);
  if (e != cudaSuccess) return bail(fail(e, "cudaEventCreate"));
  for (auto &ev : b->ev_step) {
    e = cudaEventCreate(&ev);
    if (e != cudaSuccess) return bail(fail(e, "cudaEventCreate"));
  }
  e = cudaMalloc(&b->arena, std::max<size_t>(total, 256));
  if (e != cudaSuccess) return bail(fail(e, "cudaMalloc(arena)"));
  e = cudaMalloc(reinterpret_cast<void **>(&b->dtraj), sizeof(TrajDev) * ntraj + sizeof(double) * STAT_N * ntraj +
                                                        sizeof(int) * (ntraj + kCounters));
  if (e != cudaSuccess) return bail(fail(e, "cudaMalloc(traj)"));
  b->dstats = reinterpret_cast<double *>(b->dtraj + ntraj);
  b->dstatus = reinterpret_cast<int *>(b->dstats + STAT_N * ntraj);
  b->dcounter = b->dstatus + ntraj;
  for (uint32_t i = 0; i < ntraj; ++i) {
    TrajDev &d = b->h[i];
    char *base = reinterpret_cast<char *>(b->arena) + off[i];
    const uint32_t c = b->cap[i], n = ns[i];
    d.gamma = base;
    d.lam = reinterpret_cast<double *>(base + align256(size_t(2) * c * c * eb * n));
    d.chi = reinterpret_cast<int *>(reinterpret_cast<char *>(d.lam) + align256(sizeof(double) * size_t(c) * (n + 1)));
    d.status = b->dstatus + i;
    d.stats = b->dstats + size_t(STAT_N) * i;
    d.n = int(n);
    d.cap = int(c);
    if (truncs) {
      d.trunc_mode = truncs[i].mode;
      d.chi_max = int(std::min<uint32_t>(truncs[i].chi_max, 0x7fffffff));
      d.cutoff = truncs[i].cutoff;
    } else {
      d.trunc_mode = TN_TRUNC_NONE;
      d.chi_max = 0;
      d.cutoff = 0.0;
    }
  }
  e = cudaMemcpyAsync(b->dtraj, b->h.data(), sizeof(TrajDev) * ntraj, cudaMemcpyHostToDevice, b->st);
  if (e == cudaSuccess) e = cudaMemsetAsync(b->dstatus, 0, sizeof(int) * (ntraj + 8), b->st);
  if (e == cudaSuccess) e = cudaMemsetAsync(b->dstats, 0, sizeof(double) * STAT_N * ntraj, b->st);
  if (e != cudaSuccess) return bail(fail(e, "init"));
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, dev);
  b->sortP = next_pow2(2 * b->maxcap);
  b->bps = run_blocks_per_sm(precision, b->sortP);
  b->grid_max = std::max(1, b->sms * b->bps);
  b->grid_max = std::min<int>(b->grid_max, int(std::max<uint32_t>(ntraj, b->sum_n / 2)));
  b->ws_stride = run_work_bytes(precision, b->maxcap);
  e = cudaMalloc(&b->ws, b->ws_stride * b->grid_max);
  if (e != cudaSuccess) return bail(fail(e, "cudaMalloc(workspace)"));
  b->pcap = 4 * b->maxn + 8;
  // reset all slots to |0...0>
  std::vector<int> all(ntraj);
  std::iota(all.begin(), all.end(), 0);
  int *dlist = nullptr;
  e = cudaMalloc(&dlist, sizeof(int) * ntraj);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dlist, all.data(), sizeof(int) * ntraj, cudaMemcpyHostToDevice, b->st);
  if (e == cudaSuccess) e = launch_reset(b->dtraj, dlist, int(ntraj), precision, b->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->st);
  if (dlist) cudaFree(dlist);
  if (e != cudaSuccess) return bail(fail(e, "reset"));
  *out = b;
  return TN_OK;
}

int tn_batch_free(tn_batch *b) {
  if (!b) return TN_OK;
  if (b->st) cudaStreamSynchronize(b->st);
  for (auto &kv : b->graphs) cudaGraphExecDestroy(kv.second);
  if (b->din) cudaFree(b->din);
  if (b->dprog) cudaFree(b->dprog);
  if (b->dstep) cudaFree(b->dstep);
  if (b->hstep) cudaFreeHost(b->hstep);
  if (b->ws) cudaFree(b->ws);
  if (b->dtraj) cudaFree(b->dtraj);
  if (b->arena) cudaFree(b->arena);
  for (auto &ev : b->ev)
    if (ev) cudaEventDestroy(ev);
  if (b->ev_done) cudaEventDestroy(b->ev_done);
  for (auto &ev : b->ev_step)
    if (ev) cudaEventDestroy(ev);
  if (b->st) cudaStreamDestroy(b->st);
  delete b;
  return TN_OK;
}

int tn_batch_reset(tn_batch *b, uint32_t t, uint32_t n, const tn_trunc *trunc) {
  if (!b || t >= b->ntraj) return TN_ERR_INVALID_ARG;
  if (n == 0) return TN_ERR_EMPTY_SYSTEM;
  if (n > b->n_alloc[t]) return TN_ERR_CAPACITY;
  TrajDev &d = b->h[t];
  uint32_t want = trunc && (trunc->mode == TN_TRUNC_CONST || trunc->mode == TN_TRUNC_BOTH)
                      ? std::min(std::max<uint32_t>(1, trunc->chi_max), max_rank(n))
                      : std::min<uint32_t>(max_rank(n), 256);
  if (want > b->cap[t]) return TN_ERR_CAPACITY;
  d.n = int(n);
  if (trunc) {
    d.trunc_mode = trunc->mode;
    d.chi_max = int(std::min<uint32_t>(trunc->chi_max, 0x7fffffff));
    d.cutoff = trunc->cutoff;
  } else {
    d.trunc_mode = TN_TRUNC_NONE;
    d.chi_max = 0;
    d.cutoff = 0.0;
  }
  CKB(cudaMemcpyAsync(b->dtraj + t, &d, sizeof(TrajDev), cudaMemcpyHostToDevice, b->st));
  int *dl = b->dcounter + 1;
  int tt = int(t);
  CKB(cudaMemcpyAsync(dl, &tt, sizeof(int), cudaMemcpyHostToDevice, b->st));
  CKB(launch_reset(b->dtraj, dl, 1, b->prec, b->st));
  CKB(cudaStreamSynchronize(b->st));
  return TN_OK;
}

int tn_batch_import(tn_batch *b, uint32_t t, uint32_t n, const uint32_t *chi, const double *gammas, const double *lams,
                    const tn_trunc *trunc) {
  if (!b || t >= b->ntraj || (n && (!chi || !gammas || (n > 1 && !lams)))) return TN_ERR_INVALID_ARG;
  if (n == 0) return TN_ERR_EMPTY_SYSTEM;
  if (n > b->n_alloc[t]) return TN_ERR_CAPACITY;
  if (trunc && (trunc->mode < TN_TRUNC_NONE || trunc->mode > TN_TRUNC_BOTH)) return TN_ERR_INVALID_ARG;
  if (chi[0] != 1 || chi[n] != 1) return TN_ERR_STATE_SHAPE;
  size_t ng = 0, nl = 0;
  for (uint32_t k = 0; k < n; ++k) {
    if (chi[k + 1] == 0) return TN_ERR_STATE_SHAPE;
    if (chi[k + 1] > b->cap[t]) return TN_ERR_CAPACITY;
    ng += size_t(chi[k]) * 2 * chi[k + 1];
    if (k + 1 < n) nl += chi[k + 1];
  }
  for (size_t i = 0; i < 2 * ng; ++i)
    if (!std::isfinite(gammas[i])) return TN_ERR_INVALID_ARG;
  for (size_t i = 0; i < nl; ++i)
    if (!std::isfinite(lams[i])) return TN_ERR_INVALID_ARG;
  // an earlier asynchronous step may still be running on this batch
  CKB(cudaStreamSynchronize(b->st));
  TrajDev &d = b->h[t];
  d.n = int(n);
  if (trunc) {
    d.trunc_mode = trunc->mode;
    d.chi_max = int(std::min<uint32_t>(trunc->chi_max, 0x7fffffff));
    d.cutoff = trunc->cutoff;
  } else {
    d.trunc_mode = TN_TRUNC_NONE;
    d.chi_max = 0;
    d.cutoff = 0.0;
  }
  const size_t eb = prec_elem_bytes(b->prec);
  const size_t slot = size_t(2) * d.cap * d.cap * eb;
  std::vector<char> tmp;
  size_t go = 0, lo = 0;
  for (uint32_t k = 0; k < n; ++k) {
    const size_t cnt = size_t(chi[k]) * 2 * chi[k + 1];
    char *dst = static_cast<char *>(d.gamma) + slot * k;
    if (b->prec == TN_PREC_F64) {
      CKB(cudaMemcpy(dst, gammas + 2 * go, cnt * 16, cudaMemcpyHostToDevice));
    } else {
      tmp.resize(cnt * eb);
      reals_to_layout(b->prec, gammas + 2 * go, 2 * cnt, tmp.data());
      CKB(cudaMemcpy(dst, tmp.data(), tmp.size(), cudaMemcpyHostToDevice));
    }
    go += cnt;
    if (k + 1 < n) {
      CKB(cudaMemcpy(d.lam + size_t(k + 1) * d.cap, lams + lo, sizeof(double) * chi[k + 1], cudaMemcpyHostToDevice));
      lo += chi[k + 1];
    }
  }
  const double one = 1.0;
  CKB(cudaMemcpy(d.lam, &one, sizeof(double), cudaMemcpyHostToDevice));
  CKB(cudaMemcpy(d.lam + size_t(n) * d.cap, &one, sizeof(double), cudaMemcpyHostToDevice));
  std::vector<int> ichi(chi, chi + n + 1);
  CKB(cudaMemcpy(d.chi, ichi.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice));
  CKB(cudaMemcpy(b->dtraj + t, &d, sizeof(TrajDev), cudaMemcpyHostToDevice));
  return TN_OK;
}

int tn_batch_export_gamma(tn_batch *b, uint32_t t, uint32_t k, double *out, uint64_t cap, uint32_t dims[3]) {
  if (!b || t >= b->ntraj) return TN_ERR_INVALID_ARG;
  const TrajDev &d = b->h[t];
  if (k >= uint32_t(d.n)) return TN_NONE;
  CKB(cudaStreamSynchronize(b->st));
  int c[2] = {0, 0};
  CKB(cudaMemcpy(c, d.chi + k, sizeof(int) * 2, cudaMemcpyDeviceToHost));
  if (dims) {
    dims[0] = uint32_t(c[0]);
    dims[1] = 2;
    dims[2] = uint32_t(c[1]);
  }
  if (!out) return TN_OK;
  const size_t cnt = size_t(c[0]) * 2 * c[1];
  if (cap < 2 * cnt) return TN_ERR_INVALID_ARG;
  const size_t eb = prec_elem_bytes(b->prec);
  const char *src = static_cast<const char *>(d.gamma) + size_t(2) * d.cap * d.cap * eb * k;
  if (b->prec == TN_PREC_F64) {
    CKB(cudaMemcpy(out, src, cnt * 16, cudaMemcpyDeviceToHost));
  } else {
    std::vector<char> tmp(cnt * eb);
    CKB(cudaMemcpy(tmp.data(), src, tmp.size(), cudaMemcpyDeviceToHost));
    layout_to_reals(b->prec, tmp.data(), 2 * cnt, out);
  }
  return TN_OK;
}

int tn_batch_step(tn_batch *b, const uint32_t *trajs, uint32_t nt, const uint32_t *gate_off, const uint32_t *gate_ks,
                  const double *gates, const uint32_t *meas_off, const uint32_t *meas_ks, const double *us,
                  int32_t *outcomes, double *probs, double *entropy) {
  return tn_batch_step_post(b, trajs, nt, gate_off, gate_ks, gates, meas_off, meas_ks, us, nullptr, outcomes, probs,
                            entropy);
}

int tn_batch_step_post(tn_batch *b, const uint32_t *trajs, uint32_t nt, const uint32_t *gate_off,
                       const uint32_t *gate_ks, const double *gates, const uint32_t *meas_off,
                       const uint32_t *meas_ks, const double *us, const int32_t *posts, int32_t *outcomes,
                       double *probs, double *entropy) {
  if (!b || !trajs || !gate_off || !meas_off) return TN_ERR_INVALID_ARG;
  if (nt == 0) return TN_OK;
  const uint32_t ng = gate_off[nt], nm = meas_off[nt];
  if ((ng && (!gate_ks || !gates)) || (nm && (!meas_ks || !us))) return TN_ERR_INVALID_ARG;
  for (uint32_t i = 0; i < nt; ++i) {
    if (trajs[i] >= b->ntraj) return TN_ERR_INVALID_ARG;
    if (gate_off[i + 1] < gate_off[i] || meas_off[i + 1] < meas_off[i]) return TN_ERR_INVALID_ARG;
    const uint32_t n = uint32_t(b->h[trajs[i]].n);
    for (uint32_t j = meas_off[i]; j < meas_off[i + 1]; ++j) {
      if (meas_ks[j] >= n) return TN_ERR_INVALID_ARG;
      if (j > meas_off[i] && meas_ks[j] <= meas_ks[j - 1]) return TN_ERR_INVALID_ARG;
    }
  }
  // non-finite gate entries or uniforms are refused before any device work
  for (size_t j = 0; j < size_t(ng) * 32; ++j)
    if (!std::isfinite(gates[j])) return TN_ERR_INVALID_ARG;
  for (uint32_t j = 0; j < nm; ++j)
    if (!std::isfinite(us[j])) return TN_ERR_INVALID_ARG;
  int need = 8;
  for (uint32_t i = 0; i < nt; ++i)
    need = std::max<int>(need, int(gate_off[i + 1] - gate_off[i]) + int(meas_off[i + 1] - meas_off[i]) +
                                   2 * b->h[trajs[i]].n + 4);
  if (need > b->pcap) {  // grow the per-trajectory program capacity
    b->pcap = need;
    b->step_nt = 0;
  }
  // an earlier asynchronous step may still be reading the pinned block
  if (b->async_step) CKB(cudaEventSynchronize(b->ev_done));
  if (int s = ensure_step(b, nt, ng, nm)) return s;
  StepLayout L = step_layout(b->step_nt, b->step_ng, b->step_nm);
  char *hb = reinterpret_cast<char *>(b->hstep);
  int *lst = reinterpret_cast<int *>(hb + L.list);
  int *go = reinterpret_cast<int *>(hb + L.goff);
  int *mo = reinterpret_cast<int *>(hb + L.moff);
  for (uint32_t i = 0; i < nt; ++i) lst[i] = int(trajs[i]);
  for (uint32_t i = 0; i <= nt; ++i) {
    go[i] = int(gate_off[i]);
    mo[i] = int(meas_off[i]);
  }
  int *gk = reinterpret_cast<int *>(hb + L.gks);
  int *mk = reinterpret_cast<int *>(hb + L.mks);
  for (uint32_t j = 0; j < ng; ++j) gk[j] = int(gate_ks[j]);
  for (uint32_t j = 0; j < nm; ++j) mk[j] = int(meas_ks[j]);
  if (ng) std::memcpy(hb + L.gates, gates, sizeof(double) * 32 * ng);
  if (nm) std::memcpy(hb + L.us, us, sizeof(double) * nm);
  if (posts && nm) std::memcpy(hb + L.posts, posts, sizeof(int) * nm);
  if (int s = tune_before(b)) return s;
  CKB(cudaMemcpyAsync(b->dstep, b->hstep, L.in_bytes, cudaMemcpyHostToDevice, b->st));
  StepPtrs P = ptrs_of(L, reinterpret_cast<char *>(b->dstep));
  P.order = nullptr;  // ranked on the device from the current bond dimensions
  P.posts = posts ? reinterpret_cast<const int *>(reinterpret_cast<char *>(b->dstep) + L.posts) : nullptr;
  const bool step_ev = b->ev_step[0] && b->ev_step[1];  // (not created for the server's engines)
  if (step_ev) CKB(cudaEventRecord(b->ev_step[0], b->st));
  if (int s = launch_step(b, nt, P)) return s;
  if (step_ev) {
    CKB(cudaEventRecord(b->ev_step[1], b->st));
    b->ev_step_recorded = true;
  }
  const size_t out_bytes = L.total - L.out_off;
  CKB(cudaMemcpyAsync(hb + L.out_off, reinterpret_cast<char *>(b->dstep) + L.out_off, out_bytes,
                      cudaMemcpyDeviceToHost, b->st));
  CKB(cudaEventRecord(b->ev_done, b->st));
  b->pending_nt = nt;
  b->pending_nm = nm;
  if (!outcomes && !probs && !entropy && b->async_step) return TN_OK;  // collected by batch_step_collect
  return tn::batch_step_collect(b, outcomes, probs, entropy);
}

int tn_batch_device_inputs(tn_batch *b, uint32_t max_gates, uint32_t max_meas, void **d_trajs, void **d_gate_off,
                           void **d_gate_ks, void **d_gates, void **d_meas_off, void **d_meas_ks, void **d_us,
                           void **d_outcomes, void **d_probs, void **d_entropy) {
  if (!b) return TN_ERR_INVALID_ARG;
  if (b->din) {
    cudaFree(b->din);
    b->din = nullptr;
    for (auto &kv : b->graphs) cudaGraphExecDestroy(kv.second);
    b->graphs.clear();
  }
  if (int s = ensure_step(b, b->ntraj, max_gates, max_meas)) return s;
  StepLayout L = step_layout(b->ntraj, max_gates, max_meas);
  CKB(cudaMalloc(&b->din, L.total));
  b->din_gates = max_gates;
  b->din_meas = max_meas;
  char *d = reinterpret_cast<char *>(b->din);
  if (d_trajs) *d_trajs = d + L.list;
  if (d_gate_off) *d_gate_off = d + L.goff;
  if (d_gate_ks) *d_gate_ks = d + L.gks;
  if (d_gates) *d_gates = d + L.gates;
  if (d_meas_off) *d_meas_off = d + L.moff;
  if (d_meas_ks) *d_meas_ks = d + L.mks;
  if (d_us) *d_us = d + L.us;
  if (d_outcomes) *d_outcomes = d + L.outc;
  if (d_probs) *d_probs = d + L.probs;
  if (d_entropy) *d_entropy = d + L.ents;
  return TN_OK;
}

int tn_batch_step_device(tn_batch *b, uint32_t nt) {
  if (!b || !b->din || nt > b->ntraj) return TN_ERR_INVALID_ARG;
  if (nt == 0) return TN_OK;
  StepLayout L = step_layout(b->ntraj, b->din_gates, b->din_meas);
  auto it = b->graphs.find(nt);
  if (it == b->graphs.end()) {
    cudaGraph_t g = nullptr;
    cudaGraphExec_t ge = nullptr;
    CKB(cudaStreamBeginCapture(b->st, cudaStreamCaptureModeThreadLocal));
    StepPtrs P = ptrs_of(L, reinterpret_cast<char *>(b->din));
    P.order = nullptr;  // ranked on the device inside the graph
    int s = launch_step(b, nt, P, false);
    cudaError_t e = cudaStreamEndCapture(b->st, &g);
    if (s != TN_OK) {
      if (g) cudaGraphDestroy(g);
      return s;
    }
    if (e != cudaSuccess) return fail(e, "cudaStreamEndCapture");
    e = cudaGraphInstantiate(&ge, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return fail(e, "cudaGraphInstantiate");
    it = b->graphs.emplace(nt, ge).first;
  }
  CKB(cudaGraphLaunch(it->second, b->st));
  return TN_OK;
}

int tn_batch_step_ptrs(tn_batch *b, uint32_t nt, const void *d_trajs, const void *d_order, const void *d_gate_off,
                       const void *d_gate_ks, const void *d_gates, const void *d_meas_off, const void *d_meas_ks,
                       const void *d_us, void *d_outcomes, void *d_probs, void *d_entropy) {
  if (!b || nt > b->ntraj || !d_trajs || !d_gate_off || !d_meas_off || !d_entropy)
    return TN_ERR_INVALID_ARG;
  if (nt == 0) return TN_OK;
  if (int s = ensure_step(b, b->ntraj, 1, 1)) return s;
  StepPtrs P;
  P.list = static_cast<const int *>(d_trajs);
  P.order = static_cast<const int *>(d_order);
  P.goff = static_cast<const int *>(d_gate_off);
  P.gks = static_cast<const int *>(d_gate_ks);
  P.moff = static_cast<const int *>(d_meas_off);
  P.mks = static_cast<const int *>(d_meas_ks);
  P.gates = static_cast<const double *>(d_gates);
  P.us = static_cast<const double *>(d_us);
  P.outc = static_cast<int *>(d_outcomes);
  P.probs = static_cast<double *>(d_probs);
  P.ents = static_cast<double *>(d_entropy);
  if (int s = tune_before(b)) return s;
  return launch_step(b, nt, P);
}

int tn_batch_stats(tn_batch *b, double *out, int32_t reset) {
  if (!b) return TN_ERR_INVALID_ARG;
  std::vector<double> v(size_t(STAT_N) * b->ntraj);
  CKB(cudaMemcpyAsync(v.data(), b->dstats, sizeof(double) * v.size(), cudaMemcpyDeviceToHost, b->st));
  if (reset) CKB(cudaMemsetAsync(b->dstats, 0, sizeof(double) * v.size(), b->st));
  CKB(cudaStreamSynchronize(b->st));
  if (out) {
    for (int j = 0; j < STAT_N; ++j) out[j] = 0.0;
    for (uint32_t t = 0; t < b->ntraj; ++t)
      for (int j = 0; j < STAT_N; ++j) out[j] += v[size_t(t) * STAT_N + j];
  }
  return TN_OK;
}

int tn_batch_synchronize(tn_batch *b) {
  if (!b) return TN_ERR_INVALID_ARG;
  CKB(cudaStreamSynchronize(b->st));
  return TN_OK;
}

int tn_batch_bond_dims(tn_batch *b, uint32_t t, uint32_t *out, uint32_t cap) {
  if (!b || t >= b->ntraj || !out) return TN_ERR_INVALID_ARG;
  const TrajDev &d = b->h[t];
  if (d.n < 2) return TN_NONE;
  if (cap < uint32_t(d.n - 1)) return TN_ERR_INVALID_ARG;
  std::vector<int> chi(d.n + 1);
  CKB(cudaMemcpyAsync(chi.data(), d.chi, sizeof(int) * (d.n + 1), cudaMemcpyDeviceToHost, b->st));
  CKB(cudaStreamSynchronize(b->st));
  for (int i = 0; i < d.n - 1; ++i) out[i] = uint32_t(chi[i + 1]);
  return TN_OK;
}

int tn_batch_svals(tn_batch *b, uint32_t t, uint32_t bond, double *out, uint32_t cap, uint32_t *len) {
  if (!b || t >= b->ntraj) return TN_ERR_INVALID_ARG;
  const TrajDev &d = b->h[t];
  if (d.n < 2 || bond >= uint32_t(d.n - 1)) return TN_NONE;
  int l = 0;
  CKB(cudaMemcpyAsync(&l, d.chi + bond + 1, sizeof(int), cudaMemcpyDeviceToHost, b->st));
  CKB(cudaStreamSynchronize(b->st));
  if (len) *len = uint32_t(l);
  if (!out) return TN_OK;
  if (cap < uint32_t(l)) return TN_ERR_INVALID_ARG;
  CKB(cudaMemcpyAsync(out, d.lam + size_t(bond + 1) * d.cap, sizeof(double) * l, cudaMemcpyDeviceToHost, b->st));
  CKB(cudaStreamSynchronize(b->st));
  return TN_OK;
}

int tn_batch_device_status(tn_batch *b, int32_t *status) {
  if (!b || !status) return TN_ERR_INVALID_ARG;
  std::vector<int> v(b->ntraj + kCounters);
  CKB(cudaMemcpyAsync(v.data(), b->dstatus, sizeof(int) * (b->ntraj + kCounters), cudaMemcpyDeviceToHost, b->st));
  CKB(cudaMemsetAsync(b->dstatus, 0, sizeof(int) * b->ntraj, b->st));
  CKB(cudaMemsetAsync(b->dcounter + 9, 0, sizeof(int), b->st));
  CKB(cudaStreamSynchronize(b->st));
  int acc = v[b->ntraj + 9] ? ST_QUEUE_WAIT : 0;
  for (uint32_t i = 0; i < b->ntraj; ++i) acc |= v[i];
  *status = acc;
  return TN_OK;
}

int tn_batch_slot_bytes(tn_batch *b, uint32_t t, uint64_t *bytes) {
  if (!b || t >= b->ntraj || !bytes) return TN_ERR_INVALID_ARG;
  *bytes = b->slot_bytes[t];
  return TN_OK;
}

int tn_batch_autotune(tn_batch *b, uint32_t trial_steps) {
  if (!b) return TN_ERR_INVALID_ARG;
  tn_batch::Tuner &T = b->tune;
  T.on = trial_steps > 0;
  T.pending = false;
  T.trial = int(std::max<uint32_t>(trial_steps, 1));
  T.cand = 0;
  T.in_cand = 0;
  T.score.assign(kTuneCands, 0.0);
  return TN_OK;
}

int tn_batch_tuning(tn_batch *b, int32_t *cfg, double *scores) {
  if (!b || !cfg) return TN_ERR_INVALID_ARG;
  cfg[0] = b->schedule;
  cfg[1] = b->scheme;
  cfg[2] = b->theta_simt;
  cfg[3] = b->tune.on ? 1 : 0;
  if (scores)
    for (int c = 0; c < kTuneCands; ++c) scores[c] = c < int(b->tune.score.size()) ? b->tune.score[c] : 0.0;
  return TN_OK;
}

int tn_batch_set_theta_path(tn_batch *b, int32_t simt) {
  if (!b || simt < 0 || simt > 1) return TN_ERR_INVALID_ARG;
  for (auto &kv : b->graphs) cudaGraphExecDestroy(kv.second);
  b->graphs.clear();
  b->theta_simt = simt;
  return TN_OK;
}

int tn_batch_set_schedule(tn_batch *b, int32_t schedule) {
  if (!b || schedule < 0 || schedule > 1) return TN_ERR_INVALID_ARG;
  for (auto &kv : b->graphs) cudaGraphExecDestroy(kv.second);  // captured launches follow the old schedule
  b->graphs.clear();
  b->schedule = schedule;
  return TN_OK;
}

int tn_batch_set_tuning(tn_batch *b, int32_t scheme, int32_t max_sweeps) {
  if (!b || scheme < 0 || scheme > 3 || max_sweeps < 1 || max_sweeps > 200) return TN_ERR_INVALID_ARG;
  for (auto &kv : b->graphs) cudaGraphExecDestroy(kv.second);  // captured launches carry the old values
  b->graphs.clear();
  b->scheme = scheme;
  b->max_sweeps = max_sweeps;
  return TN_OK;
}

int tn_batch_last_launch_ms(tn_batch *b, float *gate_ms, float *sweep_ms) {
  if (!b) return TN_ERR_INVALID_ARG;
  if (!b->ev_recorded) return TN_NONE;
  CKB(cudaEventSynchronize(b->ev[2]));
  float g = 0.f, w = 0.f;
  CKB(cudaEventElapsedTime(&g, b->ev[0], b->ev[1]));
  if (!b->ev_one_launch) CKB(cudaEventElapsedTime(&w, b->ev[1], b->ev[2]));
  if (gate_ms) *gate_ms = g;
  if (sweep_ms) *sweep_ms = w;
  return TN_OK;
}

int tn_batch_set_queue_wait(tn_batch *b, uint64_t wait_ns, uint32_t phantom_sweeps) {
  if (!b) return TN_ERR_INVALID_ARG;
  b->queue_wait_ns = wait_ns;
  b->phantom_sweeps = phantom_sweeps;
  for (auto &kv : b->graphs) cudaGraphExecDestroy(kv.second);  // captured with the old settings
  b->graphs.clear();
  return TN_OK;
}

int tn_batch_last_step_device_ms(tn_batch *b, float *ms) {
  if (!b || !ms) return TN_ERR_INVALID_ARG;
  if (!b->ev_step_recorded) return TN_NONE;
  CKB(cudaEventSynchronize(b->ev_step[1]));
  CKB(cudaEventElapsedTime(ms, b->ev_step[0], b->ev_step[1]));
  return TN_OK;
}

int tn_batch_stream(tn_batch *b, void **stream) {
  if (!b || !stream) return TN_ERR_INVALID_ARG;
  *stream = reinterpret_cast<void *>(b->st);
  return TN_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Engine mode for the serving loop: a batch whose slots own no memory.  The
// caller (tn_serve.cpp) binds a slot to state memory it manages, uses the
// ordinary step entry points on the bound slots, and rebinds the slot when
// the request completes.
namespace tn {

tn_batch *batch_engine_create(uint32_t slots, int prec, int ws_cap, int max_n, int grid_limit, int *status) {
  *status = TN_OK;
  if (slots == 0 || ws_cap < 1 || max_n < 1) {
    *status = TN_ERR_INVALID_ARG;
    return nullptr;
  }
  tn_batch *b = new tn_batch();
  b->prec = prec;
  b->ntraj = slots;
  b->n_alloc.assign(slots, uint32_t(max_n));
  b->cap.assign(slots, uint32_t(ws_cap));
  b->h.assign(slots, TrajDev{});
  b->slot_bytes.assign(slots, 0);
  b->maxcap = ws_cap;
  b->maxn = max_n;
  b->sum_n = slots * 2;
  auto bail = [&](int s) {
    tn_batch_free(b);
    *status = s;
    return static_cast<tn_batch *>(nullptr);
  };
  cudaError_t e = cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking);
  if (e != cudaSuccess) return bail(fail(e, "cudaStreamCreate"));
  for (auto &ev : b->ev) {
    e = cudaEventCreate(&ev);
    if (e != cudaSuccess) return bail(fail(e, "cudaEventCreate"));
  }
  e = cudaEventCreateWithFlags(&b->ev_done, cudaEventDisableTiming);
  if (e != cudaSuccess) return bail(fail(e, "cudaEventCreate"));
  b->async_step = true;
  b->grid_limit = grid_limit;
  e = cudaMalloc(reinterpret_cast<void **>(&b->dtraj),
                 sizeof(TrajDev) * slots + sizeof(double) * STAT_N * slots + sizeof(int) * (slots + kCounters));
  if (e != cudaSuccess) return bail(fail(e, "cudaMalloc(traj)"));
  b->dstats = reinterpret_cast<double *>(b->dtraj + slots);
  b->dstatus = reinterpret_cast<int *>(b->dstats + STAT_N * slots);
  b->dcounter = b->dstatus + slots;
  e = cudaMemsetAsync(b->dtraj, 0,
                      sizeof(TrajDev) * slots + sizeof(double) * STAT_N * slots + sizeof(int) * (slots + kCounters),
                      b->st);
  if (e != cudaSuccess) return bail(fail(e, "init"));
  for (uint32_t i = 0; i < slots; ++i) {
    b->h[i].status = b->dstatus + i;
    b->h[i].stats = b->dstats + size_t(STAT_N) * i;
  }
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, dev);
  b->sortP = next_pow2(2 * b->maxcap);
  b->bps = run_blocks_per_sm(prec, b->sortP);
  b->grid_max = std::max(1, b->sms * b->bps);
  if (grid_limit > 0) b->grid_max = std::min(b->grid_max, grid_limit);
  b->ws_stride = run_work_bytes(prec, b->maxcap);
  e = cudaMalloc(&b->ws, b->ws_stride * b->grid_max);
  if (e != cudaSuccess) return bail(fail(e, "cudaMalloc(workspace)"));
  b->pcap = 4 * max_n + 8;
  e = cudaStreamSynchronize(b->st);
  if (e != cudaSuccess) return bail(fail(e, "init"));
  return b;
}

// Bind slot t to the state memory in d (gamma/lam/chi, n, cap, truncation)
// and reset it to |0...0>.  Stream-ordered; no synchronisation.
int batch_bind(tn_batch *b, uint32_t t, const TrajDev &d) {
  if (!b || t >= b->ntraj || d.cap > b->maxcap || d.n < 1) return TN_ERR_INVALID_ARG;
  TrajDev &h = b->h[t];
  h.gamma = d.gamma;
  h.lam = d.lam;
  h.chi = d.chi;
  h.n = d.n;
  h.cap = d.cap;
  h.trunc_mode = d.trunc_mode;
  h.chi_max = d.chi_max;
  h.cutoff = d.cutoff;
  b->n_alloc[t] = uint32_t(d.n);
  b->cap[t] = uint32_t(d.cap);
  b->maxn = std::max(b->maxn, d.n);
  CKB(cudaMemcpyAsync(b->dtraj + t, &h, sizeof(TrajDev), cudaMemcpyHostToDevice, b->st));
  int *dl = b->dcounter + 4 + (t & 3);  // small staging words, distinct per pending bind
  int tt = int(t);
  CKB(cudaMemcpyAsync(dl, &tt, sizeof(int), cudaMemcpyHostToDevice, b->st));
  CKB(launch_reset(b->dtraj, dl, 1, b->prec, b->st));
  return TN_OK;
}

cudaStream_t batch_stream(tn_batch *b) { return b->st; }

// Outputs of the last host-input step: waits for it, then copies from pinned memory.
int batch_step_collect(tn_batch *b, int32_t *outcomes, double *probs, double *entropy) {
  CKB(cudaEventSynchronize(b->ev_done));
  StepLayout L = step_layout(b->step_nt, b->step_ng, b->step_nm);
  const char *hb = reinterpret_cast<const char *>(b->hstep);
  if (outcomes && b->pending_nm) std::memcpy(outcomes, hb + L.outc, sizeof(int) * b->pending_nm);
  if (probs && b->pending_nm) std::memcpy(probs, hb + L.probs, sizeof(double) * b->pending_nm);
  if (entropy && b->pending_nt) std::memcpy(entropy, hb + L.ents, sizeof(double) * b->pending_nt);
  return TN_OK;
}

// true when the last host-input step has finished on the device
bool batch_step_done(tn_batch *b) { return cudaEventQuery(b->ev_done) == cudaSuccess; }

}  // namespace tn
