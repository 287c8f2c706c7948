// tn_serve.cpp -- continuous-batching trajectory server.
//
// Requests (one seeded Haar brickwork trajectory each: n, truncation, p,
// depth) arrive over time.  A request is admitted when a slot is free and
// its projected state footprint (n * cap^2 * 2 complex values + Lambdas)
// fits in the HBM arena; admission is first come, first served.  Each tick
// runs one persistent layer launch (tn_batch_step) over every admitted
// request -- requests of different n and chi_max share the launch -- then
// retires the requests that reached their depth, freeing their arena range
// and slot for the next admission.  State stays resident on the device for a
// request's whole life.  Latency = completion time - arrival time on the
// server clock.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <deque>
#include <map>
#include <string>
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
};

}  // namespace

struct tn_server {
  tn_batch *b = nullptr;
  int prec = TN_PREC_MIXED;
  uint32_t slots = 0, max_chi = 1, max_n = 1;
  void *arena = nullptr;
  size_t arena_bytes = 0;
  Arena alloc;
  std::deque<Pending> pending;
  std::vector<Active> act;
  std::vector<uint32_t> free_slots;
  std::deque<tn_result> done;
  uint64_t next_id = 1;
  double layers_done = 0, busy_s = 0, ticks = 0, admitted = 0, completed = 0;
  std::chrono::steady_clock::time_point t0;
  // per-tick staging
  std::vector<uint32_t> trajs, goff, gks, moff, mks;
  std::vector<double> gates, us, probs, ents;
  std::vector<int32_t> outc;
  double now() const { return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count(); }
};

namespace {

size_t footprint(const tn_server *s, const tn_request &r, uint32_t cap) {
  const size_t eb = s->prec == TN_PREC_F64 ? 16 : 8;
  return align256(size_t(2) * cap * cap * eb * r.n) + align256(sizeof(double) * size_t(cap) * (r.n + 1)) +
         align256(sizeof(int) * (r.n + 1));
}

int admit(tn_server *s) {
  while (!s->pending.empty() && !s->free_slots.empty()) {
    const Pending &p = s->pending.front();
    const uint32_t cap = cap_of(p.r);
    const size_t bytes = footprint(s, p.r, cap);
    size_t off = 0;
    if (!s->alloc.alloc(bytes, &off)) break;  // first come, first served: wait for memory
    const uint32_t slot = s->free_slots.back();
    s->free_slots.pop_back();
    TrajDev d{};
    char *base = static_cast<char *>(s->arena) + off;
    const size_t eb = s->prec == TN_PREC_F64 ? 16 : 8;
    d.gamma = base;
    d.lam = reinterpret_cast<double *>(base + align256(size_t(2) * cap * cap * eb * p.r.n));
    d.chi = reinterpret_cast<int *>(reinterpret_cast<char *>(d.lam) + align256(sizeof(double) * size_t(cap) * (p.r.n + 1)));
    d.n = int(p.r.n);
    d.cap = int(cap);
    d.trunc_mode = p.r.trunc.mode;
    d.chi_max = int(std::min<uint32_t>(p.r.trunc.chi_max, 0x7fffffff));
    d.cutoff = p.r.trunc.cutoff;
    if (int st = batch_bind(s->b, slot, d)) {
      s->alloc.release(off, bytes);
      s->free_slots.push_back(slot);
      return st;
    }
    Active &a = s->act[slot];
    a.on = true;
    a.id = p.id;
    a.r = p.r;
    a.t_arrival = p.t_arrival;
    a.t_admit = s->now();
    a.layer = 0;
    a.off = off;
    a.bytes = bytes;
    a.entropy = 0;
    s->admitted += 1;
    s->pending.pop_front();
  }
  return TN_OK;
}

}  // namespace

extern "C" {

int tn_server_create(uint64_t hbm_bytes, uint32_t max_slots, int32_t precision, uint32_t max_chi, uint32_t max_n,
                     tn_server **out) {
  if (!out || hbm_bytes == 0 || max_slots == 0 || max_chi == 0 || max_n == 0) return TN_ERR_INVALID_ARG;
  if (precision != TN_PREC_F64 && precision != TN_PREC_MIXED) return TN_ERR_INVALID_ARG;
  *out = nullptr;
  int cnt = 0;
  if (cudaGetDeviceCount(&cnt) != cudaSuccess || cnt == 0) return TN_ERR_NO_DEVICE;
  tn_server *s = new tn_server();
  s->prec = precision;
  s->slots = max_slots;
  s->max_chi = max_chi;
  s->max_n = max_n;
  int st = TN_OK;
  s->b = batch_engine_create(max_slots, precision, int(max_chi), int(max_n), 0, &st);
  if (!s->b) {
    delete s;
    return st;
  }
  cudaError_t e = cudaMalloc(&s->arena, size_t(hbm_bytes));
  if (e != cudaSuccess) {
    tn_batch_free(s->b);
    delete s;
    set_last_error("cudaMalloc(serving arena)", e);
    return TN_ERR_OOM;
  }
  s->arena_bytes = size_t(hbm_bytes);
  s->alloc.init(s->arena_bytes);
  s->act.assign(max_slots, Active{});
  for (uint32_t i = 0; i < max_slots; ++i) s->free_slots.push_back(max_slots - 1 - i);
  s->t0 = std::chrono::steady_clock::now();
  *out = s;
  return TN_OK;
}

int tn_server_free(tn_server *s) {
  if (!s) return TN_OK;
  if (s->b) tn_batch_free(s->b);
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
  s->pending.push_back(p);
  return TN_OK;
}

int tn_server_tick(tn_server *s, uint32_t *n_active, uint32_t *n_done) {
  if (!s) return TN_ERR_INVALID_ARG;
  const double t_start = s->now();
  if (int st = admit(s)) return st;
  s->trajs.clear();
  s->goff.assign(1, 0);
  s->moff.assign(1, 0);
  s->gks.clear();
  s->mks.clear();
  s->gates.clear();
  s->us.clear();
  std::vector<uint32_t> gk(256), mk(256);
  std::vector<double> g(32 * 128), u(256);
  for (uint32_t i = 0; i < s->slots; ++i) {
    Active &a = s->act[i];
    if (!a.on) continue;
    const uint32_t n = a.r.n;
    if (gk.size() < n) {
      gk.resize(n);
      mk.resize(n);
      u.resize(n);
      g.resize(32 * (n / 2 + 1));
    }
    uint32_t ng = 0, nm = 0;
    if (int st = tn_gen_layer(a.r.seed, a.r.traj, a.layer, n, a.r.p, gk.data(), g.data(), &ng, mk.data(), u.data(), &nm))
      return st;
    s->trajs.push_back(i);
    s->gks.insert(s->gks.end(), gk.begin(), gk.begin() + ng);
    s->gates.insert(s->gates.end(), g.begin(), g.begin() + 32 * size_t(ng));
    s->mks.insert(s->mks.end(), mk.begin(), mk.begin() + nm);
    s->us.insert(s->us.end(), u.begin(), u.begin() + nm);
    s->goff.push_back(uint32_t(s->gks.size()));
    s->moff.push_back(uint32_t(s->mks.size()));
  }
  const uint32_t nt = uint32_t(s->trajs.size());
  uint32_t ndone = 0;
  if (nt) {
    s->outc.resize(std::max<size_t>(1, s->mks.size()));
    s->probs.resize(std::max<size_t>(1, s->mks.size()));
    s->ents.resize(nt);
    const double z = 0;
    const uint32_t zu = 0;
    if (int st = tn_batch_step(s->b, s->trajs.data(), nt, s->goff.data(), s->gks.empty() ? &zu : s->gks.data(),
                               s->gates.empty() ? &z : s->gates.data(), s->moff.data(),
                               s->mks.empty() ? &zu : s->mks.data(), s->us.empty() ? &z : s->us.data(),
                               s->outc.data(), s->probs.data(), s->ents.data()))
      return st;
    const double t_end = s->now();
    for (uint32_t j = 0; j < nt; ++j) {
      Active &a = s->act[s->trajs[j]];
      a.entropy = s->ents[j];
      a.layer += 1;
      if (a.layer >= a.r.depth) {
        tn_result res{};
        res.id = a.id;
        res.layers = a.layer;
        res.final_entropy = a.entropy;
        res.latency_s = t_end - a.t_arrival;
        res.queue_s = a.t_admit - a.t_arrival;
        res.status = 0;
        s->done.push_back(res);
        s->alloc.release(a.off, a.bytes);
        a.on = false;
        s->free_slots.push_back(s->trajs[j]);
        s->completed += 1;
        ++ndone;
      }
    }
    s->layers_done += nt;
    s->busy_s += t_end - t_start;
    s->ticks += 1;
  }
  if (n_active) *n_active = nt;
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
  uint32_t active = 0;
  for (const auto &a : s->act) active += a.on ? 1 : 0;
  out[0] = s->layers_done;
  out[1] = s->busy_s;
  out[2] = s->ticks;
  out[3] = double(s->alloc.used());
  out[4] = double(s->pending.size());
  out[5] = double(active);
  out[6] = s->admitted;
  out[7] = s->completed;
  return TN_OK;
}

}  // extern "C"
