// tn_kernels.cu -- kernels of the trajectory engine and their launchers.
//
//  k_run        persistent executor: CTAs pull work items (one trajectory's
//               instruction list each) from an atomic counter and run them with
//               the device routines of tn_device.cuh.
//  k_compile    builds every trajectory's instruction list for one brickwork
//               layer on the device (apply_bilayer, circuit.rs:624-659 ->
//               apply_meas_prob_layer control flow, mps.rs:2206-2252).
//  k_reset      re-initialises trajectory slots to |0...0> (MPS::new,
//               mps.rs:370-391).
#include "tn_device.cuh"
#include "tn_internal.h"
#include "tn_tc.cuh"

namespace tn {

__device__ __forceinline__ unsigned long long global_ns() { return tc::global_ns(); }

__device__ __forceinline__ int load_acquire(const int *p) {
  int v;
  asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void store_release(int *p, int v) {
  asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Appends the sweep item of listed trajectory i to the pushed queue (one thread).
__device__ void push_sweep(Item *dyn, int *tail, const Item *sweeps, int i) {
  const int slot = atomicAdd(tail, 1);
  const Item s = sweeps[i];
  dyn[slot].traj = s.traj;
  dyn[slot].off = s.off;
  dyn[slot].len = s.len;
  store_release(&dyn[slot].aux, 1);
}

// Static schedule (la.rem == nullptr): items[0, count) in counter order.
// Dependency-driven schedule: a CTA takes a pushed sweep item when one is
// ready (claimed by compare-and-swap on the sweep head below the push tail),
// else the next gate item; once the gate items are gone it claims the next
// sweep slot and waits (bounded by kQueueWaitNs) for its push.  Every pushed
// item depends only on gate items already taken by running CTAs, so the
// waits end; a wait that runs out sets qerr and the CTA moves on.
template <typename T, int NT, int W>
__global__ void __launch_bounds__(NT, 1) k_run(LaunchArgs la, int sortP, int ws_cap) {
  extern __shared__ __align__(256) unsigned char smem[];
  __shared__ Item s_item;
  __shared__ int s_kind;  // 0 done, 1 gate / static item, 2 pushed sweep item, 3 skip
  __shared__ uint64_t s_bar;
  __shared__ uint32_t s_tmem;
  Smem<T, W> sm(smem, sortP);
  Work<T> wk = make_work<T>(reinterpret_cast<unsigned char *>(la.ws) + size_t(blockIdx.x) * la.ws_stride, ws_cap);
  const bool dd = la.rem != nullptr;
  // float: one 128 x 256 FP32 accumulator tile (theta and recovery GEMMs);
  // double-float: eight 128 x 64 level accumulators of the tensor-core update
  constexpr bool kTC = sizeof(T) == 4 || std::is_same<T, ::tn::dd>::value;
  constexpr uint32_t kTmemCols = sizeof(T) == 4 ? 256 : 512;
  if constexpr (kTC) {
    // the executor owns kTmemCols tensor-memory columns for its whole
    // life (one CTA per SM); released below on the kernel's only exit path
    if ((threadIdx.x >> 5) == 0) {
      tc::tmem_alloc(&s_tmem, kTmemCols);
      tc::tmem_relinquish();
    }
    if (threadIdx.x == 0) {
      tc::mbar_init(&s_bar, 1);
      tc::mbar_fence_init();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    sm.tmem = s_tmem;
    sm.bar = &s_bar;
    sm.phase = 0;
    sm.tc = la.theta_simt == 0;
  }
  for (;;) {
    if (threadIdx.x == 0) {
      const int G = la.nitems_dev ? *la.nitems_dev : la.nitems;
      int kind = 0, slot_i = -1;
      if (dd) {
        // A pushed sweep item that is already there goes first: the sweeps
        // are the serial chains that bound the launch, the gate items are
        // independent filler.
        int h = *reinterpret_cast<volatile int *>(la.dyn_head);
        while (h < *reinterpret_cast<volatile int *>(la.dyn_tail)) {
          const int prev = atomicCAS(la.dyn_head, h, h + 1);
          if (prev == h) {
            slot_i = h;
            break;
          }
          h = prev;
        }
      }
      if (slot_i < 0) {
        const int it = atomicAdd(la.counter, 1);
        if (it < G) {
          s_item = la.items[it];
          kind = 1;
        } else if (dd) {
          // no gate left: claim the next sweep slot and wait for its push
          const int h = atomicAdd(la.dyn_head, 1);
          if (h < la.nsweeps) slot_i = h;
        }
      }
      if (slot_i >= 0) {
        Item *slot = la.dyn + slot_i;
        const unsigned long long t0 = global_ns();
        const unsigned long long limit = la.queue_wait_ns ? la.queue_wait_ns : kQueueWaitNs;
        kind = 2;
        while (load_acquire(&slot->aux) == 0) {
          if (global_ns() - t0 > limit) {
            atomicExch(la.qerr, 1);
            kind = 3;
            break;
          }
          __nanosleep(200);
        }
        if (kind == 2) s_item = Item{slot->traj, slot->off, slot->len, 0};
      }
      s_kind = kind;
    }
    __syncthreads();
    const int kind = s_kind;
    const Item item = s_item;
    __syncthreads();
    if (kind == 0) break;
    if (kind == 3) continue;
    if (kind == 2) __threadfence();  // acquire side for every thread of the CTA
    run_program<T, NT, W>(la, (dd && kind == 1) ? la.gprog : la.prog, item, wk, sm);
    if (dd && kind == 1) {
      __threadfence();  // this thread's writes of the gate's result, visible device-wide
      __syncthreads();
      if (threadIdx.x == 0 && atomicSub(la.rem + item.aux, 1) == 1) {
        __threadfence();
        push_sweep(la.dyn, la.dyn_tail, la.sweeps, item.aux);
      }
    }
  }
  if constexpr (kTC) {
    tc::fence_before_sync();
    __syncthreads();
    if ((threadIdx.x >> 5) == 0) {
      tc::fence_after_sync();
      tc::tmem_dealloc(sm.tmem, kTmemCols);
    }
  }
}

__global__ void k_reset(TrajDev *trajs, const int *list, int count, int prec) {
  const int t = list[blockIdx.x];
  const TrajDev tr = trajs[t];
  const size_t slot = size_t(2) * tr.cap * tr.cap;
  for (int k = threadIdx.x; k < tr.n; k += blockDim.x) {
    if (prec == 0) {
      cpx<double> *g = reinterpret_cast<cpx<double> *>(tr.gamma) + size_t(k) * slot;
      g[0] = mkc<double>(1.0, 0.0);
      g[1] = mkc<double>(0.0, 0.0);
    } else if (prec == 2) {
      cpx<dd> *g = reinterpret_cast<cpx<dd> *>(tr.gamma) + size_t(k) * slot;
      g[0] = mkc<dd>(dd(1.f, 0.f), dd(0.f, 0.f));
      g[1] = mkc<dd>(dd(0.f, 0.f), dd(0.f, 0.f));
    } else {
      cpx<float> *g = reinterpret_cast<cpx<float> *>(tr.gamma) + size_t(k) * slot;
      g[0] = mkc<float>(1.f, 0.f);
      g[1] = mkc<float>(0.f, 0.f);
    }
  }
  for (int s = threadIdx.x; s <= tr.n; s += blockDim.x) {
    tr.lam[size_t(s) * tr.cap] = 1.0;
    tr.chi[s] = 1;
  }
}

// One thread per listed trajectory.  The layer's gates act on disjoint bonds
// (a brickwork layer, circuit.rs:523-563), so each becomes its own work item
// (gprog[g], gitems[g]) of the first launch, spread over all SMs; the
// measurement layer with its refactor sweep and the entropy read form the
// trajectory's program of the second launch, at prog + i * pcap, placed at
// items[order[i]] so that the executor pulls the most expensive trajectories
// first.  A trajectory whose gates overlap keeps them, in order, at the head
// of its second-launch program instead.
__global__ void k_compile(const TrajDev *trajs, const int *list, int nt, const int *order, const int *gate_off,
                          const int *gate_ks, const int *meas_off, const int *meas_ks, const int *posts, int pcap,
                          Instr *prog, Item *items, Instr *gprog, Item *gitems, int gcap, int *gcount) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0) *gcount = min(gate_off[nt], gcap);
  if (i >= nt) return;
  const int t = list[i];
  const int n = trajs[t].n;
  Instr *p = prog + size_t(i) * pcap;
  int pc = 0;
  auto emit = [&](int op, int k, int a, int b) {
    if (pc < pcap) p[pc] = Instr{op, k, a, b};
    ++pc;
  };
  const int g0 = gate_off[i], g1 = gate_off[i + 1];
  bool disjoint = true;
  for (int g = g0; g < g1 && disjoint; ++g)
    for (int h = g + 1; h < g1; ++h)
      if (abs(gate_ks[g] - gate_ks[h]) < 2) {
        disjoint = false;
        break;
      }
  for (int g = g0; g < g1; ++g) {
    const int k = gate_ks[g];
    const bool valid = n > 1 && k >= 0 && k < n - 1;
    if (g < gcap) {
      gprog[g] = (disjoint && valid) ? Instr{OP_GATE, k, g, 0} : Instr{OP_NOP, 0, 0, 0};
      gitems[g] = Item{t, g, 1, 0};
    } else if (disjoint) {
      atomicOr(trajs[t].status, ST_BAD_INSTR);
    }
    if (!disjoint && valid) emit(OP_GATE, k, g, 0);
  }
  const int m0 = meas_off[i], m1 = meas_off[i + 1];
  int last = -1;
  for (int j = m0; j < m1; ++j) {
    const int k = meas_ks[j];
    if (k < 0 || k >= n || k <= last) continue;  // host guarantees sorted unique
    if (last >= 0)
      for (int b = last; b < k; ++b) emit(OP_REFACTOR, b, 0, 0);
    emit(OP_MEAS, k, j, posts ? (posts[j] == 0 || posts[j] == 1 ? posts[j] : -1) : -1);
    last = k;
  }
  if (last >= 0) {
    for (int b = last; b < n - 1; ++b) emit(OP_REFACTOR, b, 0, 0);
    for (int b = n - 3; b >= 0; --b) emit(OP_REFACTOR, b, 0, 0);
  }
  if (n >= 2) emit(OP_ENTROPY, n / 2 - 1, i, 0);
  if (pc > pcap) {  // program did not fit: run nothing, flag the trajectory
    atomicOr(trajs[t].status, ST_BAD_INSTR);
    pc = 0;
  }
  items[order[i]] = Item{t, int(size_t(i) * pcap), pc, 0};
}

// Execution rank of every listed trajectory, most expensive first (one
// block of 1024 threads).  Cost from the current bond dimensions: the
// trajectory's critical path is its most expensive gate (gates run in
// parallel) plus, when the layer measures, its serial refactor sweep over
// every bond, each bond op ~ chi^3.  Ties keep list order; more than
// kLptMax trajectories keep list order altogether.
constexpr int kLptMax = 4096;

__global__ void __launch_bounds__(1024) k_lpt_order(const TrajDev *trajs, const int *list, int nt,
                                                    const int *meas_off, int *order) {
  extern __shared__ __align__(16) unsigned char lsm[];
  if (nt > kLptMax) {
    for (int i = threadIdx.x; i < nt; i += blockDim.x) order[i] = i;
    return;
  }
  int P = 1;
  while (P < nt) P <<= 1;
  double *key = reinterpret_cast<double *>(lsm);
  int *idx = reinterpret_cast<int *>(key + P);
  for (int i = threadIdx.x; i < P; i += blockDim.x) {
    double c = -1.0;
    if (i < nt) {
      const TrajDev tr = trajs[list[i]];
      double sweep = 0.0, gmax = 0.0;
      for (int b = 1; b < tr.n; ++b) {
        const double x = double(tr.chi[b]);
        const double x3 = x * x * x;
        sweep += x3;
        gmax = fmax(gmax, x3);
      }
      c = gmax + (meas_off[i + 1] > meas_off[i] ? sweep : 0.0);
    }
    key[i] = c;
    idx[i] = i;
  }
  __syncthreads();
  bitonic_desc<float, 1024, kBlockW>(key, idx, P);
  for (int r = threadIdx.x; r < nt; r += blockDim.x) order[idx[r]] = r;
}

// First gate-queue slot of every listed trajectory when trajectories are
// taken in `order` rank: an exclusive scan of the gate counts by rank (one
// block; scratch holds the counts by rank).  An `order` that is not a
// permutation of [0, nt) is replaced by the identity.
__global__ void k_gate_slots(int nt, const int *order, const int *gate_off, int *scratch, int *gstart) {
  __shared__ int carry, wsum[32];
  for (int i = threadIdx.x; i < nt; i += blockDim.x) scratch[i] = 0;
  __syncthreads();
  int bad = 0;
  for (int i = threadIdx.x; i < nt; i += blockDim.x) {
    const int r = order[i];
    if (r < 0 || r >= nt)
      bad = 1;
    else
      atomicAdd(scratch + r, 1);
  }
  __syncthreads();
  for (int r = threadIdx.x; r < nt; r += blockDim.x) bad |= scratch[r] != 1;
  bad = __syncthreads_or(bad);
  auto rank = [&](int i) { return bad ? i : order[i]; };
  for (int i = threadIdx.x; i < nt; i += blockDim.x) scratch[rank(i)] = gate_off[i + 1] - gate_off[i];
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int base = 0; base < nt; base += blockDim.x) {
    const int r = base + threadIdx.x;
    const int v = r < nt ? scratch[r] : 0;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) wsum[warp] = x;
    __syncthreads();
    if (warp == 0) {
      int w = lane < nw ? wsum[lane] : 0;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, w, o);
        if (lane >= o) w += y;
      }
      if (lane < nw) wsum[lane] = w;  // inclusive sums over warps
    }
    __syncthreads();
    const int excl = carry + (warp ? wsum[warp - 1] : 0) + x - v;
    __syncthreads();
    if (r < nt) scratch[r] = excl;
    if (threadIdx.x == blockDim.x - 1) carry = excl + v;
    __syncthreads();
  }
  for (int i = threadIdx.x; i < nt; i += blockDim.x) gstart[i] = scratch[rank(i)];
}

// k_compile for the dependency-driven schedule: the same instruction lists,
// with gate items at gitems[gstart[i] + j] (aux = i), the sweep program as
// sweeps[i], rem[i] = number of gate items of trajectory i; a trajectory
// without gate items has its sweep item pushed here.
__global__ void k_compile_dd(const TrajDev *trajs, const int *list, int nt, const int *gate_off, const int *gate_ks,
                             const int *meas_off, const int *meas_ks, const int *posts, int pcap, Instr *prog,
                             Item *sweeps,
                             Instr *gprog, Item *gitems, int gcap, int *gcount, const int *gstart, int *rem, Item *dyn,
                             int *dyn_tail) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0) *gcount = min(gate_off[nt], gcap);
  if (i >= nt) return;
  const int t = list[i];
  const int n = trajs[t].n;
  Instr *p = prog + size_t(i) * pcap;
  int pc = 0;
  auto emit = [&](int op, int k, int a, int b) {
    if (pc < pcap) p[pc] = Instr{op, k, a, b};
    ++pc;
  };
  const int g0 = gate_off[i], g1 = gate_off[i + 1];
  bool disjoint = true;
  for (int g = g0; g < g1 && disjoint; ++g)
    for (int h = g + 1; h < g1; ++h)
      if (abs(gate_ks[g] - gate_ks[h]) < 2) {
        disjoint = false;
        break;
      }
  int placed = 0;
  for (int g = g0; g < g1; ++g) {
    const int k = gate_ks[g];
    const bool valid = n > 1 && k >= 0 && k < n - 1;
    const int slot = gstart[i] + (g - g0);
    if (slot < gcap) {
      gprog[g < gcap ? g : slot] = (disjoint && valid) ? Instr{OP_GATE, k, g, 0} : Instr{OP_NOP, 0, 0, 0};
      gitems[slot] = Item{t, g < gcap ? g : slot, 1, i};
      ++placed;
    } else if (disjoint) {
      atomicOr(trajs[t].status, ST_BAD_INSTR);
    }
    if (!disjoint && valid) emit(OP_GATE, k, g, 0);
  }
  const int m0 = meas_off[i], m1 = meas_off[i + 1];
  int last = -1;
  for (int j = m0; j < m1; ++j) {
    const int k = meas_ks[j];
    if (k < 0 || k >= n || k <= last) continue;  // host guarantees sorted unique
    if (last >= 0)
      for (int b = last; b < k; ++b) emit(OP_REFACTOR, b, 0, 0);
    emit(OP_MEAS, k, j, posts ? (posts[j] == 0 || posts[j] == 1 ? posts[j] : -1) : -1);
    last = k;
  }
  if (last >= 0) {
    for (int b = last; b < n - 1; ++b) emit(OP_REFACTOR, b, 0, 0);
    for (int b = n - 3; b >= 0; --b) emit(OP_REFACTOR, b, 0, 0);
  }
  if (n >= 2) emit(OP_ENTROPY, n / 2 - 1, i, 0);
  if (pc > pcap) {  // program did not fit: run nothing, flag the trajectory
    atomicOr(trajs[t].status, ST_BAD_INSTR);
    pc = 0;
  }
  sweeps[i] = Item{t, int(size_t(i) * pcap), pc, 0};
  rem[i] = placed;
  if (placed == 0) {
    __threadfence();
    push_sweep(dyn, dyn_tail, sweeps, i);
  }
}

// ------------------------------------------------------------- launchers
// Dynamic shared memory limit configured for k_run<T> on the current
// device (raised on demand; set when a handle or batch is created, so that
// a stream capture of a launch finds it already in place).
template <typename T, int NT, int W>
static cudaError_t ensure_run_smem(size_t smem) {
  static int configured[64] = {0};
  int dev = 0;
  cudaGetDevice(&dev);
  int &have = configured[dev & 63];
  if (int(smem) > have) {
    cudaError_t e = cudaFuncSetAttribute(k_run<T, NT, W>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e != cudaSuccess) return e;
    have = int(smem);
  }
  return cudaSuccess;
}

template <typename T, int NT, int W>
static cudaError_t launch_run_t(const LaunchArgs &la, int grid, int sortP, int ws_cap, cudaStream_t st) {
  const size_t smem = SmemLayout<T, W>::total(sortP);
  cudaError_t e = ensure_run_smem<T, NT, W>(smem);
  if (e != cudaSuccess) return e;
  k_run<T, NT, W><<<grid, NT, smem, st>>>(la, sortP, ws_cap);
  return cudaGetLastError();
}

cudaError_t launch_run(int prec, const LaunchArgs &la, int grid, int sortP, int ws_cap, cudaStream_t st) {
  if (prec == 0) return launch_run_t<double, kThreads, kBlockW>(la, grid, sortP, ws_cap, st);
  if (prec == 2) return launch_run_t<dd, kThreads, kBlockW>(la, grid, sortP, ws_cap, st);
  return launch_run_t<float, kThreads, kBlockW>(la, grid, sortP, ws_cap, st);
}

size_t run_smem_bytes(int prec, int sortP) {
  if (prec == 0) return SmemLayout<double, kBlockW>::total(sortP);
  if (prec == 2) return SmemLayout<dd, kBlockW>::total(sortP);
  return SmemLayout<float, kBlockW>::total(sortP);
}

size_t run_work_bytes(int prec, int cap) {
  if (prec == 0) return work_bytes<double>(cap);
  if (prec == 2) return work_bytes<dd>(cap);
  return work_bytes<float>(cap);
}

int run_blocks_per_sm(int prec, int sortP) {
  int nb = 0;
  const size_t smem = run_smem_bytes(prec, sortP);
  cudaError_t e;
  if (prec == 0) {
    ensure_run_smem<double, kThreads, kBlockW>(smem);
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_run<double, kThreads, kBlockW>, kThreads, smem);
  } else if (prec == 2) {
    ensure_run_smem<dd, kThreads, kBlockW>(smem);
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_run<dd, kThreads, kBlockW>, kThreads, smem);
  } else {
    ensure_run_smem<float, kThreads, kBlockW>(smem);
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_run<float, kThreads, kBlockW>, kThreads, smem);
  }
  if (e != cudaSuccess || nb < 1) nb = 1;
  return nb;
}

cudaError_t launch_reset(TrajDev *trajs, const int *list, int count, int prec, cudaStream_t st) {
  if (count <= 0) return cudaSuccess;
  k_reset<<<count, 128, 0, st>>>(trajs, list, count, prec);
  return cudaGetLastError();
}

cudaError_t launch_compile(const TrajDev *trajs, const int *list, int nt, const int *order, const int *gate_off,
                           const int *gate_ks, const int *meas_off, const int *meas_ks, const int *posts, int pcap,
                           Instr *prog, Item *items, Instr *gprog, Item *gitems, int gcap, int *gcount,
                           cudaStream_t st) {
  if (nt <= 0) return cudaSuccess;
  k_compile<<<(nt + 127) / 128, 128, 0, st>>>(trajs, list, nt, order, gate_off, gate_ks, meas_off, meas_ks, posts,
                                              pcap, prog, items, gprog, gitems, gcap, gcount);
  return cudaGetLastError();
}

cudaError_t launch_lpt_order(const TrajDev *trajs, const int *list, int nt, const int *meas_off, int *order,
                             cudaStream_t st) {
  if (nt <= 0) return cudaSuccess;
  int P = 1;
  while (P < nt && P < kLptMax) P <<= 1;
  k_lpt_order<<<1, 1024, size_t(P) * (sizeof(double) + sizeof(int)), st>>>(trajs, list, nt, meas_off, order);
  return cudaGetLastError();
}

cudaError_t launch_compile_dd(const TrajDev *trajs, const int *list, int nt, const int *order, const int *gate_off,
                              const int *gate_ks, const int *meas_off, const int *meas_ks, const int *posts, int pcap,
                              Instr *prog, Item *sweeps, Instr *gprog, Item *gitems, int gcap, int *gcount,
                              int *gstart, int *scratch, int *rem, Item *dyn, int *dyn_tail, cudaStream_t st) {
  if (nt <= 0) return cudaSuccess;
  k_gate_slots<<<1, 1024, 0, st>>>(nt, order, gate_off, scratch, gstart);
  k_compile_dd<<<(nt + 127) / 128, 128, 0, st>>>(trajs, list, nt, gate_off, gate_ks, meas_off, meas_ks, posts, pcap,
                                                 prog, sweeps, gprog, gitems, gcap, gcount, gstart, rem, dyn,
                                                 dyn_tail);
  return cudaGetLastError();
}

}  // namespace tn
