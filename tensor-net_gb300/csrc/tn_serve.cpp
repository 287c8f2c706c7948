// tn_serve.cpp -- continuous-batching trajectory server.
//
// Requests (one seeded Haar brickwork trajectory each: n, truncation, p,
// depth) arrive over time.  A request is admitted when a slot is free and
// its projected state footprint (n * cap^2 * 2 complex values + Lambdas)
// fits in the HBM arena; within a cost class, admission is first come, first
// served, or least estimated work first (tn_server_set_policy), optionally
// under a cap on the class's resident requests.  Requests of one class share
// a layer launch (tn_batch_step) -- n and
// chi_max may differ inside it -- and the launch's duration is that of its
// most expensive member, so cheap requests are kept apart from expensive
// ones: class 0 holds requests whose bond capacity is at most `light_chi`,
// class 1 the rest.  Each class owns a batch engine with its own stream and a
// fixed share of the SMs (its CTA limit), and the classes step independently:
// a tick launches the next layer of every idle class, waits until at least
// one class finishes its layer, retires the requests that reached their
// depth (freeing arena range and slot) and relaunches that class at once.
// State stays resident on the device for a request's whole life.
// Latency = completion time - arrival time on the server clock.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <deque>
#include <map>
#include <string>
#include <thread>
#include <vector>

#include "tn_internal.h"
#include "tn_mps.h"

using namespace tn;

namespace {

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

uint32_t max_rank(uint32_t n) { return n / 2 >= 20 ? (1u << 20) : (1u << (n / 2)); }

uint32_t cap_of(const tn_request &r) {
  if (r.trunc.mode == TN_TRUNC_CONST || r.trunc.mode == TN_TRUNC_BOTH)
    return std::min(std::max<uint32_t>(1, r.trunc.chi_max), max_rank(r.n));
  return std::min<uint32_t>(max_rank(r.n), 256);
}

// First-fit allocator over one device arena, coalescing on free.
class Arena {
 public:
  void init(size_t bytes) {
    free_.clear();
    free_[0] = bytes;
    used_ = 0;
  }
  bool alloc(size_t bytes, size_t *off) {
    bytes = align256(bytes);
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second >= bytes) {
        *off = it->first;
        const size_t rest = it->second - bytes, at = it->first + bytes;
        free_.erase(it);
        if (rest) free_[at] = rest;
        used_ += bytes;
        return true;
      }
    }
    return false;
  }
  void release(size_t off, size_t bytes) {
    bytes = align256(bytes);
    used_ -= bytes;
    auto it = free_.emplace(off, bytes).first;
    auto nx = std::next(it);
    if (nx != free_.end() && it->first + it->second == nx->first) {
      it->second += nx->second;
      free_.erase(nx);
    }
    if (it != free_.begin()) {
      auto pv = std::prev(it);
      if (pv->first + pv->second == it->first) {
        pv->second += it->second;
        free_.erase(it);
      }
    }
  }
  size_t used() const { return used_; }

 private:
  std::map<size_t, size_t> free_;
  size_t used_ = 0;
};

struct Pending {
  uint64_t id;
  tn_request r;
  double t_arrival;
};

struct Active {
  bool on = false;
  uint64_t id = 0;
  tn_request r{};
  double t_arrival = 0, t_admit = 0;
  uint32_t layer = 0;
  size_t off = 0, bytes = 0;
  double entropy = 0;
  bool cancel = false;  // retire when the layer in flight finishes
  std::vector<double> history;  // half-chain entropy after every layer
};

// One cost class: an engine (slots bound to arena memory), its queue, and
// the staging of the layer in flight.
struct Class {
  tn_batch *b = nullptr;
  uint32_t cap_max = 0;  // requests with cap_of(r) <= cap_max (and above the previous class's)
  int ctas = 0;          // CTA limit of its launches (0 = every resident CTA)
  std::deque<Pending> pending;
  std::vector<Active> act;
  std::vector<uint32_t> free_slots;
  uint32_t max_active = 0;  // 0 = every slot
  uint32_t active = 0;
  bool inflight = false;
  std::vector<uint32_t> trajs, goff, gks, moff, mks;
  std::vector<double> gates, us, ents;
  std::vector<uint32_t> gk, mk;
  std::vector<double> g, u;
  double layers = 0, launches = 0;
};

}  // namespace

struct tn_server {
  int prec = TN_PREC_MIXED;
  uint32_t slots = 0, max_chi = 1, max_n = 1;
  void *arena = nullptr;
  size_t arena_bytes = 0;
  Arena alloc;
  Class cls[2];
  int ncls = 1;
  int policy = 0;  // 0: first come, first served; 1: least estimated work first
  std::deque<tn_result> done;
  std::map<uint64_t, std::vector<double>> histories;  // retired requests' entropies, until fetched
  uint64_t next_id = 1;
  double layers_done = 0, busy_s = 0, ticks = 0, admitted = 0, completed = 0;
  std::chrono::steady_clock::time_point t0;
  double now() const { return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count(); }
};

namespace {

size_t footprint(const tn_server *s, const tn_request &r, uint32_t cap) {
  const size_t eb = prec_elem_bytes(s->prec);
  return align256(size_t(2) * cap * cap * eb * r.n) + align256(sizeof(double) * size_t(cap) * (r.n + 1)) +
         align256(sizeof(int) * (r.n + 1));
}

int class_of(const tn_server *s, const tn_request &r) {
  return (s->ncls > 1 && cap_of(r) > s->cls[0].cap_max) ? 1 : 0;
}

// Estimated work of a request: layers x bond operations per layer (n/2
// gates + about 2n refactors) x cap^3 (the SVD cost of a saturated bond).
double est_work(const tn_request &r) {
  const double c = double(cap_of(r));
  return double(r.depth) * 2.5 * double(r.n) * c * c * c;
}

size_t pick(const tn_server *s, const Class &c) {
  if (s->policy == 0) return 0;
  size_t best = 0;
  double bw = est_work(c.pending[0].r);
  for (size_t i = 1; i < c.pending.size(); ++i) {
    const double w = est_work(c.pending[i].r);
    if (w < bw) {
      bw = w;
      best = i;
    }
  }
  return best;
}

int admit(tn_server *s, Class &c) {
  while (!c.pending.empty() && !c.free_slots.empty() && (c.max_active == 0 || c.active < c.max_active)) {
    const size_t pi = pick(s, c);
    const Pending p = c.pending[pi];
    const uint32_t cap = cap_of(p.r);
    const size_t bytes = footprint(s, p.r, cap);
    size_t off = 0;
    if (!s->alloc.alloc(bytes, &off)) break;  // in policy order: wait for memory
    const uint32_t slot = c.free_slots.back();
    c.free_slots.pop_back();
    TrajDev d{};
    char *base = static_cast<char *>(s->arena) + off;
    const size_t eb = prec_elem_bytes(s->prec);
    d.gamma = base;
    d.lam = reinterpret_cast<double *>(base + align256(size_t(2) * cap * cap * eb * p.r.n));
    d.chi = reinterpret_cast<int *>(reinterpret_cast<char *>(d.lam) + align256(sizeof(double) * size_t(cap) * (p.r.n + 1)));
    d.n = int(p.r.n);
    d.cap = int(cap);
    d.trunc_mode = p.r.trunc.mode;
    d.chi_max = int(std::min<uint32_t>(p.r.trunc.chi_max, 0x7fffffff));
    d.cutoff = p.r.trunc.cutoff;
    if (int st = batch_bind(c.b, slot, d)) {
      s->alloc.release(off, bytes);
      c.free_slots.push_back(slot);
      return st;
    }
    Active &a = c.act[slot];
    a.on = true;
    a.id = p.id;
    a.r = p.r;
    a.t_arrival = p.t_arrival;
    a.t_admit = s->now();
    a.layer = 0;
    a.off = off;
    a.bytes = bytes;
    a.entropy = 0;
    a.cancel = false;
    a.history.clear();
    a.history.reserve(p.r.depth);
    s->admitted += 1;
    c.active += 1;
    c.pending.erase(c.pending.begin() + std::ptrdiff_t(pi));
  }
  return TN_OK;
}

// Admits what fits, generates the next layer of every active request of the
// class and enqueues it (outputs are collected by collect()).
int launch(tn_server *s, Class &c) {
  if (int st = admit(s, c)) return st;
  c.trajs.clear();
  c.goff.assign(1, 0);
  c.moff.assign(1, 0);
  c.gks.clear();
  c.mks.clear();
  c.gates.clear();
  c.us.clear();
  for (uint32_t i = 0; i < uint32_t(c.act.size()); ++i) {
    Active &a = c.act[i];
    if (!a.on) continue;
    const uint32_t n = a.r.n;
    if (c.gk.size() < n) {
      c.gk.resize(n);
      c.mk.resize(n);
      c.u.resize(n);
      c.g.resize(32 * (n / 2 + 1));
    }
    uint32_t ng = 0, nm = 0;
    if (int st = tn_gen_layer(a.r.seed, a.r.traj, a.layer, n, a.r.p, c.gk.data(), c.g.data(), &ng, c.mk.data(),
                              c.u.data(), &nm))
      return st;
    c.trajs.push_back(i);
    c.gks.insert(c.gks.end(), c.gk.begin(), c.gk.begin() + ng);
    c.gates.insert(c.gates.end(), c.g.begin(), c.g.begin() + 32 * size_t(ng));
    c.mks.insert(c.mks.end(), c.mk.begin(), c.mk.begin() + nm);
    c.us.insert(c.us.end(), c.u.begin(), c.u.begin() + nm);
    c.goff.push_back(uint32_t(c.gks.size()));
    c.moff.push_back(uint32_t(c.mks.size()));
  }
  const uint32_t nt = uint32_t(c.trajs.size());
  if (!nt) return TN_OK;
  const double z = 0;
  const uint32_t zu = 0;
  if (int st = tn_batch_step(c.b, c.trajs.data(), nt, c.goff.data(), c.gks.empty() ? &zu : c.gks.data(),
                             c.gates.empty() ? &z : c.gates.data(), c.moff.data(), c.mks.empty() ? &zu : c.mks.data(),
                             c.us.empty() ? &z : c.us.data(), nullptr, nullptr, nullptr))
    return st;
  c.inflight = true;
  c.launches += 1;
  return TN_OK;
}

// Frees a resident request's slot and arena range and queues its result.
void retire(tn_server *s, Class &c, uint32_t slot, int32_t status, double t_end) {
  Active &a = c.act[slot];
  tn_result res{};
  res.id = a.id;
  res.layers = a.layer;
  res.final_entropy = a.entropy;
  res.latency_s = t_end - a.t_arrival;
  res.queue_s = a.t_admit - a.t_arrival;
  res.status = status;
  s->done.push_back(res);
  s->histories[a.id] = std::move(a.history);
  a.history.clear();
  s->alloc.release(a.off, a.bytes);
  a.on = false;
  a.cancel = false;
  c.active -= 1;
  c.free_slots.push_back(slot);
}

// Reads the entropies of the finished layer and retires completed (and
// cancelled) requests.
int collect(tn_server *s, Class &c, uint32_t *ndone) {
  const uint32_t nt = uint32_t(c.trajs.size());
  c.ents.resize(std::max<uint32_t>(nt, 1));
  if (int st = batch_step_collect(c.b, nullptr, nullptr, c.ents.data())) return st;
  c.inflight = false;
  const double t_end = s->now();
  for (uint32_t j = 0; j < nt; ++j) {
    Active &a = c.act[c.trajs[j]];
    a.entropy = c.ents[j];
    a.history.push_back(a.entropy);
    a.layer += 1;
    if (a.layer >= a.r.depth) {
      retire(s, c, c.trajs[j], TN_OK, t_end);
      s->completed += 1;
      ++*ndone;
    } else if (a.cancel) {
      retire(s, c, c.trajs[j], TN_CANCELLED, t_end);
      ++*ndone;
    }
  }
  c.layers += nt;
  s->layers_done += nt;
  c.trajs.clear();
  return TN_OK;
}

uint32_t n_active(const tn_server *s) {
  uint32_t k = 0;
  for (int i = 0; i < s->ncls; ++i)
    for (const auto &a : s->cls[i].act) k += a.on ? 1 : 0;
  return k;
}

}  // namespace

extern "C" {

int tn_server_create_classes(uint64_t hbm_bytes, uint32_t max_slots, int32_t precision, uint32_t max_chi,
                             uint32_t max_n, uint32_t light_chi, uint32_t light_ctas, tn_server **out) {
  if (!out || hbm_bytes == 0 || max_slots == 0 || max_chi == 0 || max_n == 0) return TN_ERR_INVALID_ARG;
  if (precision != TN_PREC_F64 && precision != TN_PREC_MIXED && precision != TN_PREC_DF) return TN_ERR_INVALID_ARG;
  *out = nullptr;
  int cnt = 0, dev = 0, sms = 1;
  if (cudaGetDeviceCount(&cnt) != cudaSuccess || cnt == 0) return TN_ERR_NO_DEVICE;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  tn_server *s = new tn_server();
  s->prec = precision;
  s->slots = max_slots;
  s->max_chi = max_chi;
  s->max_n = max_n;
  if (light_chi == 0) light_chi = 64;
  if (light_ctas == 0) light_ctas = uint32_t(std::max(1, sms / 5));
  const bool two = light_chi < max_chi && int(light_ctas) < sms;
  s->ncls = two ? 2 : 1;
  s->cls[0].cap_max = two ? light_chi : max_chi;
  s->cls[0].ctas = two ? int(light_ctas) : 0;
  if (two) {
    s->cls[1].cap_max = max_chi;
    s->cls[1].ctas = sms - int(light_ctas);
  }
  for (int i = 0; i < s->ncls; ++i) {
    Class &c = s->cls[i];
    int st = TN_OK;
    c.b = batch_engine_create(max_slots, precision, int(c.cap_max), int(max_n), c.ctas, &st);
    if (!c.b) {
      tn_server_free(s);
      return st;
    }
    c.act.assign(max_slots, Active{});
    for (uint32_t k = 0; k < max_slots; ++k) c.free_slots.push_back(max_slots - 1 - k);
  }
  cudaError_t e = cudaMalloc(&s->arena, size_t(hbm_bytes));
  if (e != cudaSuccess) {
    s->arena = nullptr;
    tn_server_free(s);
    set_last_error("cudaMalloc(serving arena)", e);
    return TN_ERR_OOM;
  }
  s->arena_bytes = size_t(hbm_bytes);
  s->alloc.init(s->arena_bytes);
  s->t0 = std::chrono::steady_clock::now();
  *out = s;
  return TN_OK;
}

int tn_server_create(uint64_t hbm_bytes, uint32_t max_slots, int32_t precision, uint32_t max_chi, uint32_t max_n,
                     tn_server **out) {
  return tn_server_create_classes(hbm_bytes, max_slots, precision, max_chi, max_n, 0, 0, out);
}

int tn_server_free(tn_server *s) {
  if (!s) return TN_OK;
  for (int i = 0; i < 2; ++i) {
    Class &c = s->cls[i];
    if (c.b && c.inflight) batch_step_collect(c.b, nullptr, nullptr, nullptr);
    if (c.b) tn_batch_free(c.b);
  }
  if (s->arena) cudaFree(s->arena);
  delete s;
  return TN_OK;
}

int tn_server_now(const tn_server *s, double *t) {
  if (!s || !t) return TN_ERR_INVALID_ARG;
  *t = s->now();
  return TN_OK;
}

int tn_server_submit(tn_server *s, const tn_request *r, double arrival, uint64_t *id) {
  if (!s || !r) return TN_ERR_INVALID_ARG;
  if (r->n == 0) return TN_ERR_EMPTY_SYSTEM;
  if (r->n > s->max_n || cap_of(*r) > s->max_chi || r->depth == 0) return TN_ERR_CAPACITY;
  if (r->trunc.mode < TN_TRUNC_NONE || r->trunc.mode > TN_TRUNC_BOTH) return TN_ERR_INVALID_ARG;
  if (footprint(s, *r, cap_of(*r)) > s->arena_bytes) return TN_ERR_CAPACITY;
  Pending p{s->next_id++, *r, arrival < 0 ? s->now() : arrival};
  if (id) *id = p.id;
  s->cls[class_of(s, *r)].pending.push_back(p);
  return TN_OK;
}

int tn_server_tick(tn_server *s, uint32_t *n_active_out, uint32_t *n_done) {
  if (!s) return TN_ERR_INVALID_ARG;
  const double t_start = s->now();
  uint32_t ndone = 0;
  bool progress = false;
  for (;;) {
    bool any = false;
    for (int i = 0; i < s->ncls; ++i) {
      Class &c = s->cls[i];
      if (c.inflight && batch_step_done(c.b)) {
        if (int st = collect(s, c, &ndone)) return st;
        progress = true;
      }
    }
    for (int i = 0; i < s->ncls; ++i) {
      Class &c = s->cls[i];
      if (!c.inflight)
        if (int st = launch(s, c)) return st;
      any = any || c.inflight;
    }
    if (progress || !any) break;
    std::this_thread::sleep_for(std::chrono::microseconds(20));
  }
  if (progress) {
    s->busy_s += s->now() - t_start;
    s->ticks += 1;
  }
  if (n_active_out) *n_active_out = n_active(s);
  if (n_done) *n_done = ndone;
  return TN_OK;
}

int tn_server_poll(tn_server *s, tn_result *out, uint32_t cap, uint32_t *n) {
  if (!s || (cap && !out)) return TN_ERR_INVALID_ARG;
  uint32_t k = 0;
  while (k < cap && !s->done.empty()) {
    out[k++] = s->done.front();
    s->done.pop_front();
  }
  if (n) *n = k;
  return TN_OK;
}

int tn_server_stats(const tn_server *s, double *out) {
  if (!s || !out) return TN_ERR_INVALID_ARG;
  size_t pending = 0;
  for (int i = 0; i < s->ncls; ++i) pending += s->cls[i].pending.size();
  out[0] = s->layers_done;
  out[1] = s->busy_s;
  out[2] = s->ticks;
  out[3] = double(s->alloc.used());
  out[4] = double(pending);
  out[5] = double(n_active(s));
  out[6] = s->admitted;
  out[7] = s->completed;
  return TN_OK;
}

int tn_server_history(tn_server *s, uint64_t id, double *out, uint32_t cap, uint32_t *len) {
  if (!s) return TN_ERR_INVALID_ARG;
  auto it = s->histories.find(id);
  if (it == s->histories.end()) return TN_NONE;
  const uint32_t l = uint32_t(it->second.size());
  if (len) *len = l;
  if (!out) return TN_OK;
  if (cap < l) return TN_ERR_INVALID_ARG;
  std::copy(it->second.begin(), it->second.end(), out);
  s->histories.erase(it);
  return TN_OK;
}

int tn_server_cancel(tn_server *s, uint64_t id) {
  if (!s) return TN_ERR_INVALID_ARG;
  for (int i = 0; i < s->ncls; ++i) {
    Class &c = s->cls[i];
    for (size_t j = 0; j < c.pending.size(); ++j) {
      if (c.pending[j].id != id) continue;
      tn_result res{};
      res.id = id;
      res.latency_s = s->now() - c.pending[j].t_arrival;
      res.queue_s = res.latency_s;
      res.status = TN_CANCELLED;
      s->done.push_back(res);
      c.pending.erase(c.pending.begin() + std::ptrdiff_t(j));
      return TN_OK;
    }
    for (uint32_t slot = 0; slot < uint32_t(c.act.size()); ++slot) {
      Active &a = c.act[slot];
      if (!a.on || a.id != id) continue;
      if (c.inflight) {
        a.cancel = true;  // its layer is running: retired by collect()
      } else {
        retire(s, c, slot, TN_CANCELLED, s->now());
      }
      return TN_OK;
    }
  }
  return TN_NONE;
}

int tn_server_set_policy(tn_server *s, int32_t policy, uint32_t max_active0, uint32_t max_active1) {
  if (!s || policy < 0 || policy > 1) return TN_ERR_INVALID_ARG;
  s->policy = policy;
  s->cls[0].max_active = max_active0;
  s->cls[1].max_active = max_active1;
  return TN_OK;
}

int tn_server_class_stats(const tn_server *s, uint32_t cls, double *out) {
  if (!s || !out || cls >= 2) return TN_ERR_INVALID_ARG;
  for (int i = 0; i < 6; ++i) out[i] = 0;
  if (int(cls) >= s->ncls) return TN_OK;
  const Class &c = s->cls[cls];
  uint32_t active = 0;
  for (const auto &a : c.act) active += a.on ? 1 : 0;
  out[0] = double(c.cap_max);
  out[1] = double(c.ctas);
  out[2] = c.layers;
  out[3] = c.launches;
  out[4] = double(c.pending.size());
  out[5] = double(active);
  return TN_OK;
}

}  // extern "C"
