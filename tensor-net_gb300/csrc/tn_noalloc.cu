// tn_noalloc.cu -- apply_unitary2 without any device allocation.
//
// Some callers cannot allocate device memory at the point where they apply a
// gate: a host runtime that reserves its whole device budget up front and
// forbids allocation afterwards (a serving loop with a fixed memory plan, a
// Rust caller inside a no-allocation section), or code that runs while other
// work on the device is being captured into a CUDA graph, where an
// allocation would be illegal or would break the capture.  For them,
// tn_mps_apply_unitary2_noalloc does what tn_mps_apply_unitary2 does, but
// the bond operation's scratch (theta, the Jacobi vectors, the per-value
// factors) lives in a fixed, file-scope device array instead of the handle's
// workspace, and the one-instruction program, its work item, the gate matrix
// and the work-queue counter live in small fixed device arrays too.  Nothing
// is allocated per call; the arrays exist once per GPU that loads the library
// and stay until the process exits.
//
// Limits and sharing:
//  - the scratch holds kScratchBytes (4.5 MiB): enough for a bond capacity
//    of chi <= 270 in mixed precision (so every chi_max <= 256 of the
//    workloads) and chi <= 191 in float64 or double-float; larger handles
//    are rejected with TN_ERR_CAPACITY before anything is launched;
//  - the gate is refused with TN_ERR_INVALID_ARG when an entry is not
//    finite, before any device work, as tn_mps_apply_unitary2 does;
//  - the gate, program and work item are staged from host memory that lives
//    only during the call, so the handle's stream must not be capturing a
//    CUDA graph (checked: TN_ERR_INVALID_ARG);
//  - every call, on every stream and handle, uses the same arrays, and they
//    keep the last call's contents.  The counter is cleared by each call;
//    the scratch needs no clearing (each bond operation writes the parts it
//    reads).  Calls that overlap on the GPU (different streams, or host
//    threads racing) corrupt each other: order them on one stream;
//  - the first call on a device looks up the arrays' device addresses
//    (cudaGetSymbolAddress, with that device current); make that first call
//    before any stream capture begins.
#include <cmath>
#include <cstring>
#include <mutex>

#include "tn_internal.h"
#include "tn_mps.h"

namespace {

constexpr size_t kScratchBytes = size_t(9) << 19;  // 4.5 MiB
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];
static __device__ __align__(16) tn::Instr g_prog[1];
static __device__ __align__(16) tn::Item g_item[1];
static __device__ __align__(16) double g_gate[32];
static __device__ __align__(16) int g_counter[4];

struct DeviceSymbols {
  bool ready = false;
  void *scratch = nullptr, *prog = nullptr, *item = nullptr, *gate = nullptr, *counter = nullptr;
};

DeviceSymbols g_syms[kMaxDevices];
std::mutex g_setup;

// Looks up the device addresses of the arrays for the current device once.
int setup_current_device(DeviceSymbols **out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    tn::set_last_error("cudaGetDevice", e);
    return TN_ERR_CUDA;
  }
  if (dev < 0 || dev >= kMaxDevices) return TN_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lock(g_setup);
  DeviceSymbols &s = g_syms[dev];
  if (!s.ready) {
    struct {
      void **dst;
      const void *sym;
      const char *name;
    } table[] = {{&s.scratch, reinterpret_cast<const void *>(&g_scratch), "cudaGetSymbolAddress(g_scratch)"},
                 {&s.prog, reinterpret_cast<const void *>(&g_prog), "cudaGetSymbolAddress(g_prog)"},
                 {&s.item, reinterpret_cast<const void *>(&g_item), "cudaGetSymbolAddress(g_item)"},
                 {&s.gate, reinterpret_cast<const void *>(&g_gate), "cudaGetSymbolAddress(g_gate)"},
                 {&s.counter, reinterpret_cast<const void *>(&g_counter), "cudaGetSymbolAddress(g_counter)"}};
    for (auto &t : table) {
      e = cudaGetSymbolAddress(t.dst, t.sym);
      if (e != cudaSuccess) {
        tn::set_last_error(t.name, e);
        return TN_ERR_CUDA;
      }
    }
    s.ready = true;
  }
  *out = &s;
  return TN_OK;
}

}  // namespace

extern "C" int tn_mps_apply_unitary2_noalloc(tn_mps *m, uint32_t k, const double *op, uint32_t rows, uint32_t cols) {
  if (!m || !op) return TN_ERR_INVALID_ARG;
  tn::MpsView v;
  if (int s = tn::mps_view(m, &v)) return s;
  // argument handling identical to tn_mps_apply_unitary2 (mps.rs:1332-1341)
  if (v.n == 1 || k >= uint32_t(v.n - 1)) return TN_OK;
  if (rows != 4 || cols != 4) return TN_ERR_OPERATOR_SHAPE;
  for (int i = 0; i < 32; ++i)
    if (!std::isfinite(op[i])) return TN_ERR_INVALID_ARG;
  const size_t need = tn::run_work_bytes(v.prec, v.cap);
  if (need > kScratchBytes) {
    tn::set_last_error("tn_mps_apply_unitary2_noalloc: the handle's bond capacity needs more scratch than the "
                       "4.5 MiB fixed array (chi <= 270 in mixed precision, chi <= 191 in float64 or double-float)",
                       cudaSuccess);
    return TN_ERR_CAPACITY;
  }
  cudaStreamCaptureStatus cap_status = cudaStreamCaptureStatusNone;
  cudaError_t ce = cudaStreamIsCapturing(v.st, &cap_status);
  if (ce != cudaSuccess) {
    tn::set_last_error("tn_mps_apply_unitary2_noalloc: cudaStreamIsCapturing", ce);
    return TN_ERR_CUDA;
  }
  if (cap_status != cudaStreamCaptureStatusNone) return TN_ERR_INVALID_ARG;
  DeviceSymbols *s = nullptr;
  if (int st = setup_current_device(&s)) return st;
  const tn::Instr prog{tn::OP_GATE, int(k), 0, 0};
  const tn::Item item{0, 0, 1, 0};
  cudaError_t e = cudaMemcpyAsync(s->gate, op, 32 * sizeof(double), cudaMemcpyHostToDevice, v.st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(s->prog, &prog, sizeof(prog), cudaMemcpyHostToDevice, v.st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(s->item, &item, sizeof(item), cudaMemcpyHostToDevice, v.st);
  if (e == cudaSuccess) e = cudaMemsetAsync(s->counter, 0, sizeof(int), v.st);
  if (e != cudaSuccess) {
    tn::set_last_error("tn_mps_apply_unitary2_noalloc: staging", e);
    return TN_ERR_CUDA;
  }
  tn::LaunchArgs la{};
  la.items = static_cast<const tn::Item *>(s->item);
  la.nitems = 1;
  la.counter = static_cast<int *>(s->counter);
  la.trajs = v.dtraj;
  la.prog = static_cast<const tn::Instr *>(s->prog);
  la.gates = static_cast<const double *>(s->gate);
  la.ws = s->scratch;
  la.ws_stride = 0;
  la.max_sweeps = 40;
  la.jacobi_scheme = tn::kDefaultScheme;
  e = tn::launch_run(v.prec, la, 1, tn::next_pow2(2 * v.cap), v.cap, v.st);
  if (e != cudaSuccess) {
    tn::set_last_error("tn_mps_apply_unitary2_noalloc: launch", e);
    return TN_ERR_CUDA;
  }
  return TN_OK;
}
