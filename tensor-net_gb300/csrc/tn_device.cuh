// tn_device.cuh -- device side of the Gamma-Lambda MPS trajectory engine (sm_103a).
//
// One CTA owns one trajectory for the whole of a launch and executes that
// trajectory's instruction list (gates, refactors, measurements, entropy reads)
// in order.  Trajectory state stays in HBM between launches:
//   gamma : n slots of 2*cap*cap complex<T>; site k holds Gamma_k as a dense
//           row-major (chi_{k-1}, 2, chi_k) array at the slot start (the
//           reference layout, tensor-net/lib/mps.rs:344-349);
//   lam   : n+1 slots of cap float64; slot 0 and slot n hold [1.0] so that the
//           chain-end branches of the reference collapse into one formula,
//           slot b+1 holds Lambda_b (mps.rs:352-353);
//   chi   : n+1 ints, chi[b+1] = dim of bond b, chi[0] = chi[n] = 1.
// A bond operation on (k, k+1) follows local_refactor / apply_unitary2
// (mps.rs:846-880, 1332-1387): theta build -> one-sided Jacobi SVD -> sort,
// truncate, renormalise (process_svd, mps.rs:236-293) -> Gamma rebuild and
// local_renormalize (mps.rs:1147-1209).
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

#include "tn_dd.cuh"
#include "tn_internal.h"
#include "tn_tc.cuh"

namespace tn {

// ---------------------------------------------------------------- complex
template <typename T>
struct __align__(2 * sizeof(T)) cpx {
  T x, y;
};

template <typename T>
__device__ __forceinline__ cpx<T> mkc(T x, T y) {
  cpx<T> r;
  r.x = x;
  r.y = y;
  return r;
}
template <typename T>
__device__ __forceinline__ cpx<T> czero() {
  return mkc<T>(T(0), T(0));
}
template <typename T>
__device__ __forceinline__ cpx<T> cadd(cpx<T> a, cpx<T> b) {
  return mkc<T>(a.x + b.x, a.y + b.y);
}
template <typename T>
__device__ __forceinline__ cpx<T> cmul(cpx<T> a, cpx<T> b) {
  return mkc<T>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
template <typename T>
__device__ __forceinline__ cpx<T> cscale(cpx<T> a, T s) {
  return mkc<T>(a.x * s, a.y * s);
}
// acc + a*b
template <typename T>
__device__ __forceinline__ cpx<T> cfma(cpx<T> a, cpx<T> b, cpx<T> acc) {
  acc.x = fma(a.x, b.x, acc.x);
  acc.x = fma(-a.y, b.y, acc.x);
  acc.y = fma(a.x, b.y, acc.y);
  acc.y = fma(a.y, b.x, acc.y);
  return acc;
}
// acc + conj(a)*b
template <typename T>
__device__ __forceinline__ cpx<T> cjfma(cpx<T> a, cpx<T> b, cpx<T> acc) {
  acc.x = fma(a.x, b.x, acc.x);
  acc.x = fma(a.y, b.y, acc.x);
  acc.y = fma(a.x, b.y, acc.y);
  acc.y = fma(-a.y, b.x, acc.y);
  return acc;
}
template <typename T>
__device__ __forceinline__ T cabs2(cpx<T> a) {
  return a.x * a.x + a.y * a.y;
}

template <typename T>
struct Eps;
template <>
struct Eps<double> {
  static constexpr double v = 2.220446049250313e-16;
};
template <>
struct Eps<float> {
  static constexpr float v = 1.1920929e-07f;
};
// rounding unit of the double-float operations (2^-47: the low float's own
// rounding and the uncompensated cross terms of a product)
template <>
struct Eps<dd> {
  static constexpr double v = 7.105427357601002e-15;
};

// Relative size (to ||A||_F = ||s||) below which a singular value is rounding
// noise of the working precision: such vectors are neither rotated by the
// Jacobi sweeps nor kept by the rank rule.  float and double: the rounding
// level of a computed Gram entry (the rank rule uses 2 sqrt(ell) eps32 /
// 4 sqrt(ell) eps64; the sweeps skip vectors below eps ||A||).  dd: the same
// 4 sqrt(ell) eps rule, but never below 1e-12: the double-float pair has
// float32's exponent range, so the Gram entries of vectors below that size
// (|a_p||a_q| * tol < 1e-37) would reach float32's subnormal range and
// could no longer be resolved to the tolerance.
template <typename T>
__host__ __device__ inline double rank_floor(int ell) {
  return (sizeof(T) == 4 ? 2.0 : 4.0) * sqrt(double(ell)) * double(Eps<T>::v);
}
template <>
__host__ __device__ inline double rank_floor<dd>(int ell) {
  const double f = 4.0 * sqrt(double(ell)) * Eps<dd>::v;
  return f > 1e-12 ? f : 1e-12;
}
template <typename T>
__host__ __device__ inline double sweep_floor(int) {
  return double(Eps<T>::v);
}
template <>
__host__ __device__ inline double sweep_floor<dd>(int ell) {
  return rank_floor<dd>(ell);
}

// Accumulators of sums of complex products.  For float and double the
// accumulator is the complex value itself and acc_fin is the identity (the
// arithmetic is exactly cfma / cjfma); for dd it is a pair of raw
// accumulators (dacc) normalised once by acc_fin after the loop.
template <typename T>
struct CAcc {
  using type = cpx<T>;
};
struct cdacc {
  dacc x, y;
};
template <>
struct CAcc<dd> {
  using type = cdacc;
};
template <typename T>
__device__ __forceinline__ typename CAcc<T>::type acc_zero() {
  return czero<T>();
}
template <>
__device__ __forceinline__ cdacc acc_zero<dd>() {
  cdacc a;
  a.x.hi = a.x.lo = a.y.hi = a.y.lo = 0.f;
  return a;
}
// acc + a*b
template <typename T>
__device__ __forceinline__ void acc_fma(typename CAcc<T>::type &acc, cpx<T> a, cpx<T> b) {
  acc = cfma(a, b, acc);
}
template <>
__device__ __forceinline__ void acc_fma<dd>(cdacc &acc, cpx<dd> a, cpx<dd> b) {
  dacc_add_prod(acc.x, a.x, b.x);
  dacc_add_prod(acc.x, -a.y, b.y);
  dacc_add_prod(acc.y, a.x, b.y);
  dacc_add_prod(acc.y, a.y, b.x);
}
// acc + conj(a)*b
template <typename T>
__device__ __forceinline__ void acc_jfma(typename CAcc<T>::type &acc, cpx<T> a, cpx<T> b) {
  acc = cjfma(a, b, acc);
}
template <>
__device__ __forceinline__ void acc_jfma<dd>(cdacc &acc, cpx<dd> a, cpx<dd> b) {
  dacc_add_prod(acc.x, a.x, b.x);
  dacc_add_prod(acc.x, a.y, b.y);
  dacc_add_prod(acc.y, a.x, b.y);
  dacc_add_prod(acc.y, -a.y, b.x);
}
template <typename T>
__device__ __forceinline__ cpx<T> acc_fin(const typename CAcc<T>::type &acc) {
  return acc;
}
template <>
__device__ __forceinline__ cpx<dd> acc_fin<dd>(const cdacc &acc) {
  return mkc<dd>(dd_norm(acc.x.hi, acc.x.lo), dd_norm(acc.y.hi, acc.y.lo));
}

// --------------------------------------------------------- block helpers
template <int NT>
__device__ __forceinline__ double block_sum(double v, double *red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  if (warp == 0) {
    double t = (lane < NT / 32) ? red[lane] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if (lane == 0) red[32] = t;
  }
  __syncthreads();
  return red[32];
}

template <int NT>
__device__ __forceinline__ void block_sum2(double &a, double &b, double *red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, o);
    b += __shfl_xor_sync(0xffffffffu, b, o);
  }
  __syncthreads();
  if (lane == 0) {
    red[warp] = a;
    red[32 + warp] = b;
  }
  __syncthreads();
  if (warp == 0) {
    double t = (lane < NT / 32) ? red[lane] : 0.0;
    double u = (lane < NT / 32) ? red[32 + lane] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      t += __shfl_xor_sync(0xffffffffu, t, o);
      u += __shfl_xor_sync(0xffffffffu, u, o);
    }
    if (lane == 0) {
      red[64] = t;
      red[65] = u;
    }
  }
  __syncthreads();
  a = red[64];
  b = red[65];
}

template <int NT>
__device__ __forceinline__ int block_min_int(int v, int *red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, o));
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  if (warp == 0) {
    int t = (lane < NT / 32) ? red[lane] : 0x7fffffff;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t = min(t, __shfl_xor_sync(0xffffffffu, t, o));
    if (lane == 0) red[32] = t;
  }
  __syncthreads();
  return red[32];
}

// ------------------------------------------------------- shared layout
// W = vectors per Jacobi block pair (two blocks of W/2).  The float path keeps
// the block pair resident in shared memory when vectors have at most
// RES_ROWS elements; otherwise (and for float64) it is streamed from L2 in
// 32-row chunks.
template <typename T, int W>
struct SmemLayout {
  static constexpr int TU = 16;
  static constexpr int TILE = 32;                 // theta tile: 32 (v) x 32 (w)
  static constexpr int TP = W + 1;                // padded row pitch of Ts
  // row pitch of the resident block Ab: even for float, so that a row starts
  // on a 16-byte boundary and the Gram's broadcast reads are 16 bytes wide
  static constexpr int AP = sizeof(T) == 4 ? W + 2 : W + 1;
  static constexpr int RES_ROWS = sizeof(T) == 4 ? 512 : 0;
  static constexpr int GK = 16, GT = 64;          // recovery GEMM: K chunk, 64x64 tile
  static constexpr size_t theta_bytes = size_t(2) * TILE * 2 * TU * sizeof(cpx<T>);
  static constexpr size_t gemm_bytes = size_t(2) * GK * (GT + 1) * sizeof(cpx<T>);
  __host__ __device__ static size_t sort_bytes(int P) { return size_t(P) * (sizeof(double) + sizeof(int)); }
  __host__ __device__ static size_t region0(int P) {
    size_t g = theta_bytes > gemm_bytes ? theta_bytes : gemm_bytes, s = sort_bytes(P);
    size_t r = g > s ? g : s;
    return (r + 255) & ~size_t(255);
  }
  static constexpr size_t ab_bytes = size_t(RES_ROWS) * AP * sizeof(cpx<T>);
  static constexpr int GP = W + 1;                // padded row pitch of G and J
  static constexpr size_t g_bytes = size_t(W) * GP * sizeof(cpx<T>);
  static constexpr size_t ts_bytes = size_t(32) * TP * sizeof(cpx<T>);
  // double-float executor: staging of the block update on the tensor cores
  // (OzUpdate): digit planes of a 128-row x 32 K-chunk of the block and of
  // the 64 x 64 real rotation, plus per-row / per-column exponents
  static constexpr int OZ_DIGITS = 8, OZ_MT = 128, OZ_KC = 32, OZ_N = 64;
  static constexpr size_t oz_a_plane = size_t(OZ_MT) * OZ_KC * 2, oz_b_plane = size_t(OZ_N) * OZ_N * 2;
  static constexpr size_t oz_bytes = std::is_same<T, dd>::value
                                         ? OZ_DIGITS * (oz_a_plane + oz_b_plane) + 4 * OZ_MT * sizeof(float) +
                                               (OZ_MT + OZ_N + W) * sizeof(int)
                                         : 0;
  __host__ __device__ static size_t total(int P) {
    return region0(P) + ab_bytes + 2 * g_bytes + ts_bytes + 128 * sizeof(double) + 256 * sizeof(int) + 512 +
           (oz_bytes ? oz_bytes + 1024 : 0);
  }
};

template <typename T, int W>
struct Smem {
  unsigned char *r0;
  cpx<T> *Ab, *G, *J, *Ts;  // G and J: W x W, row pitch W + 1
  double *red;
  int *ired;
  // tensor-core state of the CTA (float executor): accumulator columns in
  // tensor memory, the MMA-completion mbarrier and its phase
  uint64_t *bar = nullptr;
  uint32_t tmem = 0, phase = 0;
  bool tc = false;
  bool tc_fail = false;  // an MMA wait ran past its limit during the current bond op
  unsigned char *oz = nullptr;  // double-float executor: tensor-core update staging (1024-byte aligned)
  __device__ Smem(unsigned char *base, int P) {
    using L = SmemLayout<T, W>;
    auto al = [](unsigned char *q) {
      return reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(q) + 15) & ~uintptr_t(15));
    };
    unsigned char *p = base;
    r0 = p;
    p += L::region0(P);
    Ab = reinterpret_cast<cpx<T> *>(p);
    p += L::ab_bytes;
    G = reinterpret_cast<cpx<T> *>(p);
    p += L::g_bytes;
    J = reinterpret_cast<cpx<T> *>(p);
    p += L::g_bytes;
    Ts = reinterpret_cast<cpx<T> *>(p);
    p += L::ts_bytes;
    p = al(p);
    red = reinterpret_cast<double *>(p);
    p += 128 * sizeof(double);
    ired = reinterpret_cast<int *>(p);
    p += 256 * sizeof(int);
    if (L::oz_bytes) oz = reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(p) + 1023) & ~uintptr_t(1023));
  }
};

// ------------------------------------------------------------- workspace
// Per-CTA global scratch (L2-resident for the CTA's current bond operation).
template <typename T>
struct Work {
  cpx<T> *A;     // Jacobi vectors, vector-contiguous, up to 4*cap^2
  cpx<T> *T0;    // copy of theta in the same layout (for the recovered side)
  double *sig;   // 2*cap singular values, sorted descending
  double *s2;    // 2*cap kept Schmidt values
  T *scl;        // 2*cap row/column scale factors
  int *perm;     // 2*cap source vector of each kept value
  T *lam3;       // 3*cap: Lambda_{k-1}, Lambda_k, Lambda_{k+1} in the working precision
  T *isig;       // 2*cap: 1/sigma_j and (after cap*2) 1/sigma_j^2 of the kept values
  T *isig2;
  T *w2;         // 2*cap: s2_j^2 in the working precision
};

template <typename T>
__host__ __device__ inline size_t work_bytes(int cap) {
  size_t n4 = size_t(4) * cap * cap;
  size_t b = 2 * n4 * sizeof(cpx<T>) + size_t(4) * cap * sizeof(double) + size_t(2) * cap * sizeof(T) +
             size_t(2) * cap * sizeof(int) + size_t(3) * cap * sizeof(T) + size_t(6) * cap * sizeof(T) + 256;
  return (b + 255) & ~size_t(255);
}

template <typename T>
__device__ inline Work<T> make_work(void *base, int cap) {
  Work<T> w;
  unsigned char *p = reinterpret_cast<unsigned char *>(base);
  size_t n4 = size_t(4) * cap * cap;
  w.A = reinterpret_cast<cpx<T> *>(p);
  p += n4 * sizeof(cpx<T>);
  w.T0 = reinterpret_cast<cpx<T> *>(p);
  p += n4 * sizeof(cpx<T>);
  w.sig = reinterpret_cast<double *>(p);
  p += size_t(2) * cap * sizeof(double);
  w.s2 = reinterpret_cast<double *>(p);
  p += size_t(2) * cap * sizeof(double);
  w.scl = reinterpret_cast<T *>(p);
  p += size_t(2) * cap * sizeof(T);
  w.perm = reinterpret_cast<int *>(p);
  p += size_t(2) * cap * sizeof(int);
  p = reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(p) + 15) & ~uintptr_t(15));
  w.lam3 = reinterpret_cast<T *>(p);
  p += size_t(3) * cap * sizeof(T);
  w.isig = reinterpret_cast<T *>(p);
  p += size_t(2) * cap * sizeof(T);
  w.isig2 = reinterpret_cast<T *>(p);
  p += size_t(2) * cap * sizeof(T);
  w.w2 = reinterpret_cast<T *>(p);
  return w;
}

__device__ __forceinline__ bool is_normal_pos(double s, double eps) {
  // f64::is_normal() && s > eps  (mps.rs:254-258, 262-266)
  return isfinite(s) && s != 0.0 && fabs(s) >= 2.2250738585072014e-308 && s > eps;
}

// Round-robin (circle method) pairing: round r of W-1, pair t of W/2.
template <int W>
__device__ __forceinline__ void rr_pair(int r, int t, int &p, int &q) {
  auto pos = [&](int x) { return x == 0 ? 0 : ((x - 1 + r) % (W - 1)) + 1; };
  int a = pos(t), b = pos(W - 1 - t);
  p = a < b ? a : b;
  q = a < b ? b : a;
}

// =======================================================================
// Phase 1: theta = Lambda_{k-1} Gamma_k Lambda_k Gamma_{k+1} Lambda_{k+1},
// then op on the fused physical pair (do_contract2 mps.rs:628-651,
// contract_local2 732-754, apply_unitary2 1343-1352).
// Writes A (and its copy T0) vector-contiguous: colmode A[j*m + i] =
// theta[i][j] (vectors = columns, m > nc), else A[i*nc + j] = theta[i][j].
// =======================================================================
template <typename T, int NT, int W>
__device__ void build_theta(const cpx<T> *__restrict__ gk, const cpx<T> *__restrict__ gk1,
                            const T *__restrict__ lamL, const T *__restrict__ lamM,
                            const T *__restrict__ lamR, int cL, int cM, int cR,
                            const double *__restrict__ gate, cpx<T> *__restrict__ A, cpx<T> *__restrict__ T0,
                            bool colmode, Smem<T, W> &sm) {
  using L = SmemLayout<T, W>;
  constexpr int TILE = L::TILE, TU = L::TU;
  constexpr int PER = (TILE * TILE) / NT;  // (v,w) outputs per thread
  static_assert(PER >= 1 && (TILE * TILE) % NT == 0, "tile/threads");
  cpx<T> *Xs = reinterpret_cast<cpx<T> *>(sm.r0);  // [TILE v][2][TU]
  cpx<T> *Ys = Xs + TILE * 2 * TU;                // [TU][2][TILE w]
  const int m = 2 * cL, nc = 2 * cR;
  const int ell = colmode ? m : nc;

  cpx<T> op[16];
  if (gate) {
#pragma unroll
    for (int i = 0; i < 16; ++i) op[i] = mkc<T>(T(gate[2 * i]), T(gate[2 * i + 1]));
  }
  const int tid = threadIdx.x;
  for (int v0 = 0; v0 < cL; v0 += TILE) {
    for (int w0 = 0; w0 < cR; w0 += TILE) {
      typename CAcc<T>::type acc[PER][4];
#pragma unroll
      for (int e = 0; e < PER; ++e)
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[e][q] = acc_zero<T>();
      for (int u0 = 0; u0 < cM; u0 += TU) {
        __syncthreads();
        for (int idx = tid; idx < TILE * 2 * TU; idx += NT) {
          int u = idx % TU, s = (idx / TU) & 1, v = idx / (2 * TU);
          int gv = v0 + v, gu = u0 + u;
          cpx<T> x = czero<T>();
          if (gv < cL && gu < cM) x = gk[(size_t(gv) * 2 + s) * cM + gu];
          Xs[idx] = x;
        }
        for (int idx = tid; idx < TU * 2 * TILE; idx += NT) {
          int w = idx % TILE, s = (idx / TILE) & 1, u = idx / (2 * TILE);
          int gw = w0 + w, gu = u0 + u;
          cpx<T> y = czero<T>();
          if (gw < cR && gu < cM) y = cscale(gk1[(size_t(gu) * 2 + s) * cR + gw], lamM[gu]);
          Ys[idx] = y;
        }
        __syncthreads();
#pragma unroll
        for (int e = 0; e < PER; ++e) {
          int o = tid + e * NT;
          int v = o / TILE, w = o % TILE;
#pragma unroll 4
          for (int u = 0; u < TU; ++u) {
            cpx<T> x0 = Xs[(v * 2 + 0) * TU + u], x1 = Xs[(v * 2 + 1) * TU + u];
            cpx<T> y0 = Ys[(u * 2 + 0) * TILE + w], y1 = Ys[(u * 2 + 1) * TILE + w];
            acc_fma<T>(acc[e][0], x0, y0);
            acc_fma<T>(acc[e][1], x0, y1);
            acc_fma<T>(acc[e][2], x1, y0);
            acc_fma<T>(acc[e][3], x1, y1);
          }
        }
      }
      // epilogue: Lambda_{k-1}, Lambda_{k+1} scaling, gate on (s1 s2), store
#pragma unroll
      for (int e = 0; e < PER; ++e) {
        int o = tid + e * NT;
        int v = v0 + o / TILE, w = w0 + o % TILE;
        if (v < cL && w < cR) {
          const T sl = lamL[v], sr = lamR[w];
          cpx<T> th[4];
#pragma unroll
          for (int q = 0; q < 4; ++q) th[q] = cscale(cscale(acc_fin<T>(acc[e][q]), sl), sr);
          if (gate) {
            cpx<T> t2[4];
#pragma unroll
            for (int a = 0; a < 4; ++a) {
              cpx<T> s = czero<T>();
#pragma unroll
              for (int b = 0; b < 4; ++b) s = cfma(op[a * 4 + b], th[b], s);
              t2[a] = s;
            }
#pragma unroll
            for (int a = 0; a < 4; ++a) th[a] = t2[a];
          }
#pragma unroll
          for (int a = 0; a < 4; ++a) {
            int s1 = a >> 1, s2 = a & 1;
            int i = 2 * v + s1, j = s2 * cR + w;
            size_t o2 = colmode ? size_t(j) * ell + i : size_t(i) * ell + j;
            A[o2] = th[a];
            T0[o2] = th[a];
          }
        }
      }
    }
  }
  __syncthreads();
}

// Waits (every thread) for the MMAs committed to sm.bar; false when they did
// not complete within 10 s (the caller flags the trajectory).
template <typename T, int W>
__device__ bool wait_mma(Smem<T, W> &sm) {
  const uint64_t t0 = tc::global_ns();
  bool ok = true;
  while (!tc::mbar_try_wait(sm.bar, sm.phase)) {
    if (tc::global_ns() - t0 > 10ull * 1000 * 1000 * 1000) {
      ok = false;
      break;
    }
  }
  sm.phase ^= 1u;
  if (!ok) sm.tc_fail = true;
  return ok;
}

// theta on the tensor cores (float executor): the complex GEMM
// X (2cL x cM, Gamma_k rows) * Y (cM x 2cR, Lambda_k Gamma_{k+1}) as one real
// GEMM of the real view of X (interleaved re/im along K) with the 2x2 real
// embedding [[Yr, Yi], [-Yi, Yr]] of Y, in 128 x 256 tiles of kind::tf32
// tcgen05.mma with the accumulator in tensor memory.  Each operand is split
// into a TF32 part and its remainder (3 products: hi*hi + hi*lo + lo*hi,
// accumulated in FP32), which keeps the products to about 2^-21 relative.
// Output columns of a tile are ordered (w, s2, re/im), so one thread holds
// theta[(v, s1), (s2, w)] for both s2 of its row and its partner lane holds
// the other s1: the Lambda scaling and the 4x4 gate on (s1 s2) are applied in
// registers before the stores, as in build_theta.  Shared memory: the tiles
// live in the resident Jacobi block's area, idle while theta is built.
template <int NT, int W>
__device__ bool build_theta_tc(const cpx<float> *gk, const cpx<float> *gk1, const float *lamL, const float *lamM,
                               const float *lamR, int cL, int cM, int cR, const double *gate, cpx<float> *A,
                               cpx<float> *T0, bool colmode, Smem<float, W> &sm) {
  constexpr int MT = 128, NTL = 256, KC = 32, WT = NTL / 4;
  constexpr uint32_t IDESC = tc::idesc_tf32(MT, NTL);
  constexpr uint32_t LBO = 128, SBO = KC * 32;
  static_assert(SmemLayout<float, W>::ab_bytes >= size_t(2 * (MT + NTL) * KC) * sizeof(float), "tiles fit");
  float *Ahi = reinterpret_cast<float *>(sm.Ab), *Alo = Ahi + MT * KC, *Bhi = Alo + MT * KC, *Blo = Bhi + NTL * KC;
  const int m = 2 * cL, nc = 2 * cR, K2 = 2 * cM;
  const int ell = colmode ? m : nc;
  const float *gkf = reinterpret_cast<const float *>(gk);
  cpx<float> U[16];
  if (gate) {
#pragma unroll
    for (int q = 0; q < 16; ++q) U[q] = mkc<float>(float(gate[2 * q]), float(gate[2 * q + 1]));
  }
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  bool ok = true;
  for (int i0 = 0; i0 < m; i0 += MT) {
    for (int w0 = 0; w0 < cR; w0 += WT) {
      int chunk = 0;
      for (int k0 = 0; k0 < K2; k0 += KC, ++chunk) {
        if (chunk > 0) ok = wait_mma<float, W>(sm) && ok;  // the staging tiles are free again
        for (int idx = tid; idx < MT * KC; idx += NT) {
          // idx * 4 bytes == tc::kmajor_offset(r, k, KC)
          const int core = idx >> 5, within = idx & 31;
          const int r = (core / (KC / 4)) * 8 + (within >> 2), k = (core % (KC / 4)) * 4 + (within & 3);
          const int i = i0 + r, kk = k0 + k;
          const float x = (i < m && kk < K2) ? gkf[size_t(i) * K2 + kk] : 0.f;
          float hi, lo;
          tc::split_tf32(x, hi, lo);
          Ahi[idx] = hi;
          Alo[idx] = lo;
        }
        for (int idx = tid; idx < NTL * KC; idx += NT) {
          const int core = idx >> 5, within = idx & 31;
          const int nl = (core / (KC / 4)) * 8 + (within >> 2), k = (core % (KC / 4)) * 4 + (within & 3);
          const int kk = k0 + k, u = kk >> 1, a = kk & 1;
          const int b = nl & 1, s2 = (nl >> 1) & 1, w = w0 + (nl >> 2);
          float x = 0.f;
          if (u < cM && w < cR) {
            const cpx<float> y = gk1[size_t(u) * nc + s2 * cR + w];
            const float l = lamM[u];
            x = (a == b) ? y.x * l : (a == 0 ? y.y * l : -y.y * l);  // [[Yr, Yi], [-Yi, Yr]]
          }
          float hi, lo;
          tc::split_tf32(x, hi, lo);
          Bhi[idx] = hi;
          Blo[idx] = lo;
        }
        tc::fence_smem_to_async();
        __syncthreads();
        if (tid == 0) {
          tc::fence_after_sync();
#pragma unroll
          for (int st = 0; st < KC / 8; ++st) {
            const uint32_t off = uint32_t(st) * 2 * LBO;  // 8 K values = two core matrices
            const uint64_t ah = tc::smem_desc(reinterpret_cast<char *>(Ahi) + off, LBO, SBO);
            const uint64_t al = tc::smem_desc(reinterpret_cast<char *>(Alo) + off, LBO, SBO);
            const uint64_t bh = tc::smem_desc(reinterpret_cast<char *>(Bhi) + off, LBO, SBO);
            const uint64_t bl = tc::smem_desc(reinterpret_cast<char *>(Blo) + off, LBO, SBO);
            tc::mma_tf32(sm.tmem, ah, bh, IDESC, (chunk > 0 || st > 0) ? 1u : 0u);
            tc::mma_tf32(sm.tmem, ah, bl, IDESC, 1u);
            tc::mma_tf32(sm.tmem, al, bh, IDESC, 1u);
          }
          tc::mma_commit(sm.bar);
        }
      }
      ok = wait_mma<float, W>(sm) && ok;
      tc::fence_after_sync();
      // epilogue: warp w reads lanes 32 (w % 4) .. +31 (rows) and columns 64 (w / 4) .. +63
      const int sp = warp & 3, cq = warp >> 2;
      const int i = i0 + 32 * sp + lane;
      const int v = i >> 1, s1 = i & 1;
      const float sl = i < m ? lamL[v] : 0.f;
#pragma unroll 1
      for (int c16 = 0; c16 < 4; ++c16) {
        float d[16];
        tc::tmem_ld16(sm.tmem + (uint32_t(32 * sp) << 16) + uint32_t(64 * cq + 16 * c16), d);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int w = w0 + 16 * cq + 4 * c16 + q;
          const float sc = sl * (w < cR ? lamR[w] : 0.f);
          cpx<float> t[2] = {mkc<float>(d[4 * q] * sc, d[4 * q + 1] * sc),
                             mkc<float>(d[4 * q + 2] * sc, d[4 * q + 3] * sc)};
          cpx<float> pt[2];
#pragma unroll
          for (int s = 0; s < 2; ++s) {
            pt[s].x = __shfl_xor_sync(0xffffffffu, t[s].x, 1);
            pt[s].y = __shfl_xor_sync(0xffffffffu, t[s].y, 1);
          }
          cpx<float> out[2] = {t[0], t[1]};
          if (gate) {
            // th[(s1', s2')]: own row s1' = s1, partner row s1' = 1 - s1
            cpx<float> th[4];
            th[2 * s1] = t[0];
            th[2 * s1 + 1] = t[1];
            th[2 * (1 - s1)] = pt[0];
            th[2 * (1 - s1) + 1] = pt[1];
#pragma unroll
            for (int s = 0; s < 2; ++s) {
              cpx<float> acc = czero<float>();
#pragma unroll
              for (int bb = 0; bb < 4; ++bb) acc = cfma(U[(2 * s1 + s) * 4 + bb], th[bb], acc);
              out[s] = acc;
            }
          }
          if (i < m && w < cR) {
#pragma unroll
            for (int s = 0; s < 2; ++s) {
              const int j = s * cR + w;
              const size_t o2 = colmode ? size_t(j) * ell + i : size_t(i) * ell + j;
              A[o2] = out[s];
              T0[o2] = out[s];
            }
          }
        }
      }
      tc::fence_before_sync();
      __syncthreads();
    }
  }
  return ok;
}

// =======================================================================
// Phase 2: one-sided (Hestenes) block Jacobi on the c vectors of length ell
// stored in A (vector-contiguous).  Block pairs of W vectors: Gram matrix
// G = Ab^H Ab (W x W), one cyclic sweep of two-sided Jacobi on G with the
// round-robin parallel ordering, accumulating J, then Ab <- Ab J.  Converged
// when every pair satisfies |a_p^H a_q| <= tol |a_p| |a_q|, tol = sqrt(ell) eps.
// The rotations are not accumulated: the other singular side is recovered
// from the saved theta in the finalisation.  Returns the number of sweeps,
// or -1 when the sweep limit was hit.
// =======================================================================

// -- streamed path (float64, or float with ell > RES_ROWS) ---------------
template <typename T, int NT, int W>
__device__ void load_block_chunk(const cpx<T> *__restrict__ A, int ell, const int *cols, int i0, cpx<T> *Ts) {
  constexpr int TP = W + 1;
  for (int idx = threadIdx.x; idx < 32 * W; idx += NT) {
    int r = idx & 31, p = idx >> 5;
    cpx<T> v = czero<T>();
    if (cols[p] >= 0 && i0 + r < ell) v = A[size_t(cols[p]) * ell + i0 + r];
    Ts[r * TP + p] = v;
  }
}

template <typename T, int NT, int W>
__device__ void gram_stream(const cpx<T> *__restrict__ A, int ell, const int *cols, Smem<T, W> &sm) {
  constexpr int TP = W + 1;
  constexpr int PER = (W * W + NT - 1) / NT;
  typename CAcc<T>::type acc[PER];
#pragma unroll
  for (int e = 0; e < PER; ++e) acc[e] = acc_zero<T>();
  for (int i0 = 0; i0 < ell; i0 += 32) {
    __syncthreads();
    load_block_chunk<T, NT, W>(A, ell, cols, i0, sm.Ts);
    __syncthreads();
    const int rmax = min(32, ell - i0);
#pragma unroll
    for (int e = 0; e < PER; ++e) {
      int o = threadIdx.x + e * NT;
      if (o < W * W) {
        int p = o / W, q = o % W;
        typename CAcc<T>::type a = acc[e];
        for (int r = 0; r < rmax; ++r) acc_jfma<T>(a, sm.Ts[r * TP + p], sm.Ts[r * TP + q]);
        acc[e] = a;
      }
    }
  }
#pragma unroll
  for (int e = 0; e < PER; ++e) {
    int o = threadIdx.x + e * NT;
    if (o < W * W) sm.G[(o / W) * (W + 1) + o % W] = acc_fin<T>(acc[e]);
  }
  __syncthreads();
}

// Row p and column q (p <= q) of entry e of the upper triangle of a W x W
// matrix, row by row.
template <int W>
__device__ __forceinline__ void upper_entry(int e, int &p, int &q) {
  int r = 0, base = 0;
  while (base + (W - r) <= e) {
    base += W - r;
    ++r;
  }
  p = r;
  q = r + (e - base);
}

// Hermitian Gram of a double-float block, streamed: only the W (W + 1) / 2
// entries with p <= q are summed (G_qp = conj G_pq).  Thread t < NT sums
// upper entry t over every row; the remaining W (W + 1) / 2 - NT entries are
// summed one per warp, each lane over every 32nd row, and reduced across the
// warp at the end (double-float raw accumulators throughout).
template <int NT, int W>
__device__ void gram_stream_herm(const cpx<dd> *__restrict__ A, int ell, const int *cols, Smem<dd, W> &sm) {
  constexpr int TP = W + 1, NE = W * (W + 1) / 2, NX = NE - NT;
  static_assert(NX >= 0 && NX <= NT / 32, "one leftover entry per warp at most");
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int p0, q0, px = 0, qx = 0;
  upper_entry<W>(threadIdx.x, p0, q0);
  const bool extra = warp < NX;
  if (extra) upper_entry<W>(NT + warp, px, qx);
  cdacc acc = acc_zero<dd>(), accx = acc_zero<dd>();
  for (int i0 = 0; i0 < ell; i0 += 32) {
    __syncthreads();
    load_block_chunk<dd, NT, W>(A, ell, cols, i0, sm.Ts);
    __syncthreads();
    const int rmax = min(32, ell - i0);
    for (int r = 0; r < rmax; ++r) acc_jfma<dd>(acc, sm.Ts[r * TP + p0], sm.Ts[r * TP + q0]);
    if (extra && lane < rmax) acc_jfma<dd>(accx, sm.Ts[lane * TP + px], sm.Ts[lane * TP + qx]);
  }
  cpx<dd> g = acc_fin<dd>(acc);
  sm.G[p0 * TP + q0] = g;
  if (p0 != q0) sm.G[q0 * TP + p0] = mkc<dd>(g.x, -g.y);
  if (extra) {
    cpx<dd> gx = acc_fin<dd>(accx);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      gx.x += shfl_xor(gx.x, o);
      gx.y += shfl_xor(gx.y, o);
    }
    if (lane == 0) {
      sm.G[px * TP + qx] = gx;
      if (px != qx) sm.G[qx * TP + px] = mkc<dd>(gx.x, -gx.y);
    }
  }
  __syncthreads();
}

// Float Gram of the leading halves of double-float vectors (the guided
// sweeps of jacobi_svd<dd>): the 32-row chunks of the block's hi parts
// staged as complex float in Ts, G (complex float, row pitch W + 1) written
// over sm.G's area.  The hi parts carry each entry to float precision
// relative to that entry (2^-24), the precision the float Gram needs.
template <int NT, int W>
__device__ void gram_stream_hi(const cpx<dd> *__restrict__ A, int ell, const int *cols, Smem<dd, W> &sm) {
  constexpr int TP = W + 1;
  constexpr int PER = (W * W + NT - 1) / NT;
  cpx<float> *Ts = reinterpret_cast<cpx<float> *>(sm.Ts);
  cpx<float> *G = reinterpret_cast<cpx<float> *>(sm.G);
  cpx<float> acc[PER];
#pragma unroll
  for (int e = 0; e < PER; ++e) acc[e] = czero<float>();
  for (int i0 = 0; i0 < ell; i0 += 32) {
    __syncthreads();
    for (int idx = threadIdx.x; idx < 32 * W; idx += NT) {
      const int r = idx & 31, q = idx >> 5;
      cpx<float> v = czero<float>();
      if (cols[q] >= 0 && i0 + r < ell) {
        const cpx<dd> x = A[size_t(cols[q]) * ell + i0 + r];
        v = mkc<float>(x.x.hi, x.y.hi);
      }
      Ts[r * TP + q] = v;
    }
    __syncthreads();
    const int rmax = min(32, ell - i0);
#pragma unroll
    for (int e = 0; e < PER; ++e) {
      const int o = threadIdx.x + e * NT;
      if (o < W * W) {
        const int pp = o / W, qq = o % W;
        cpx<float> a = acc[e];
        for (int r = 0; r < rmax; ++r) a = cjfma(Ts[r * TP + pp], Ts[r * TP + qq], a);
        acc[e] = a;
      }
    }
  }
#pragma unroll
  for (int e = 0; e < PER; ++e) {
    const int o = threadIdx.x + e * NT;
    if (o < W * W) G[(o / W) * (W + 1) + o % W] = acc[e];
  }
  __syncthreads();
}

// X (rows x W slice of a vector-contiguous matrix, vector length ld) <- X J
template <typename T, int NT, int W>
__device__ void update_stream(cpx<T> *__restrict__ X, int ld, int rows, const int *cols,
                              const cpx<T> *__restrict__ Jm, Smem<T, W> &sm) {
  constexpr int TP = W + 1;
  constexpr int PER = (32 * W + NT - 1) / NT;
  for (int i0 = 0; i0 < rows; i0 += 32) {
    __syncthreads();
    load_block_chunk<T, NT, W>(X, ld, cols, i0, sm.Ts);
    __syncthreads();
    cpx<T> out[PER];
#pragma unroll
    for (int e = 0; e < PER; ++e) {
      int o = threadIdx.x + e * NT;
      out[e] = czero<T>();
      if (o < 32 * W) {
        int q = o >> 5, r = o & 31;
        if (cols[q] >= 0) {
          typename CAcc<T>::type a = acc_zero<T>();
          for (int p = 0; p < W; ++p) acc_fma<T>(a, sm.Ts[r * TP + p], Jm[p * (W + 1) + q]);
          out[e] = acc_fin<T>(a);
        }
      }
    }
#pragma unroll
    for (int e = 0; e < PER; ++e) {
      int o = threadIdx.x + e * NT;
      if (o < 32 * W) {
        int q = o >> 5, r = o & 31;
        if (cols[q] >= 0 && i0 + r < rows) X[size_t(cols[q]) * ld + i0 + r] = out[e];
      }
    }
  }
  __syncthreads();
}

// -- double-float block update on the tensor cores -----------------------
// x * 2^e (exact while the result is a normal float)
__device__ __forceinline__ float pow2f(int e) { return __int_as_float((127 + e) << 23); }
__device__ __forceinline__ float scale2f(float x, int e) {
  while (e > 126) {
    x = __fmul_rn(x, pow2f(126));
    e -= 126;
  }
  while (e < -126) {
    x = __fmul_rn(x, pow2f(-126));
    e += 126;
  }
  return __fmul_rn(x, pow2f(e));
}
// Exponent e with |v| < 2^e for every |v| <= m (m the largest magnitude of a
// row or column; 0 when m == 0).
__device__ __forceinline__ int oz_exponent(float m) {
  int e = 0;
  if (m > 0.f) frexpf(m, &e);
  return e;
}
// ND signed BITS-bit digits of the double-float x = hi + lo relative to 2^E
// (|x| < 2^E): x = 2^E sum_j d_j 2^(-BITS (j + 1)) + r,
// |r| <= 2^(E - BITS ND - 1); |d_0| <= 2^BITS, |d_j| <= 2^(BITS-1) after.
// Each digit is an integer, exact in bf16 (BITS <= 7).
template <int ND, int BITS = 7>
__device__ __forceinline__ void oz_digits(float hi, float lo, int E, float (&d)[ND]) {
  constexpr float R = float(1 << BITS);
  float rh = scale2f(hi, BITS - E), rl = scale2f(lo, BITS - E);
#pragma unroll
  for (int j = 0; j < ND; ++j) {
    d[j] = rintf(rh);
    float s, e;
    two_sum(__fsub_rn(rh, d[j]), rl, s, e);  // the remainder, exactly
    rh = __fmul_rn(s, R);
    rl = __fmul_rn(e, R);
  }
}
// Element offset in a K-major, no-swizzle bf16 tile with KC values per row:
// 8-row x 16-byte core matrices, 128 bytes apart along K, KC * 16 bytes
// apart between 8-row groups.
__device__ __forceinline__ uint32_t oz_elem(int r, int k, int KC) {
  return uint32_t((r >> 3) * (KC * 8) + (k >> 3) * 64 + (r & 7) * 8 + (k & 7));
}

// A_b <- A_b J for the 32 double-float vectors cols[0..32) of A (vector
// length ell) on the tensor cores, exact to the double-float level: an
// Ozaki-style splitting.  The block is the real ell x 64 matrix X (re/im of
// the 32 vectors interleaved) and J the real 64 x 64 embedding Y =
// [[Jr, Ji], [-Ji, Jr]].  Each vector is first divided by a power of two
// near its norm (2^-e_p, exact) and J's row p multiplied by the same 2^e_p,
// so that the entries of one row of X are of comparable size.  Each row of X
// (each column of Y) is then written relative to a power of two above its
// largest entry as 8 signed 7-bit integer digits (bf16, exact); the digit
// products of a pair (j, k) summed over the 64 K values stay below 2^21, and
// the up to 8 pairs with j + k = L (weight 2^(-7 (L + 2))) accumulate,
// exactly (below 2^22), in one FP32 tensor-memory accumulator per level
// L = 0..7 (kind::f16 MMAs, 128 x 64 x 16; 8 x 64 = 512 columns).  The
// levels are added from the largest in double-float and scaled back.
// Dropped levels (j + k >= 8) weigh below 2^-49 of the scales.  Rows go in
// tiles of 128, K in two chunks of 32 (the digit planes of a chunk:
// 8 x 8 KB).  Returns false when an MMA wait ran past its limit.
template <int NT, int W>
__device__ bool update_ozaki(cpx<dd> *__restrict__ A, int ell, const int *cols, const cpx<dd> *__restrict__ Jm,
                             const float *__restrict__ gdiag, Smem<dd, W> &sm) {
  using L = SmemLayout<dd, W>;
  constexpr int ND = L::OZ_DIGITS, MT = L::OZ_MT, KC = L::OZ_KC, NN = L::OZ_N, GP = W + 1;
  static_assert(W == 32 && NT == 512 && NN == 2 * W && 2 * KC == NN, "Ozaki update layout");
  constexpr uint32_t IDESC = tc::idesc_bf16(MT, NN);
  __nv_bfloat16 *Ap = reinterpret_cast<__nv_bfloat16 *>(sm.oz);        // ND planes of MT x KC
  __nv_bfloat16 *Bp = Ap + size_t(ND) * MT * KC;                        // ND planes of NN x NN (K = NN)
  float *rmax = reinterpret_cast<float *>(Bp + size_t(ND) * NN * NN);   // 4 x MT partial row maxima
  int *Erow = reinterpret_cast<int *>(rmax + 4 * MT);                   // MT
  int *Fcol = Erow + MT;                                                // NN
  float *vexp = reinterpret_cast<float *>(Fcol + NN);                   // W: 2^e_p near each vector's norm
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  bool ok = true;
  if (tid < W) {
    const float gd = gdiag[tid];  // the vector's squared norm (Gram diagonal before this step's rotations)
    vexp[tid] = (cols[tid] >= 0 && gd > 0.f && isfinite(gd)) ? pow2f(oz_exponent(sqrtf(gd))) : 1.f;
  }
  __syncthreads();
  // B: digit planes of diag(2^e_p) Y, column scale per output vector q
  if (tid < W) {
    float m = 0.f;
    for (int pp = 0; pp < W; ++pp) {
      const cpx<dd> j = Jm[pp * GP + tid];
      const float sc = vexp[pp];
      m = fmaxf(m, fmaxf(fabsf(j.x.hi), fabsf(j.y.hi)) * sc);
    }
    const int e = oz_exponent(m);
    Fcol[2 * tid] = e;
    Fcol[2 * tid + 1] = e;
  }
  __syncthreads();
  for (int idx = tid; idx < NN * NN; idx += NT) {  // (c, k): output column c, K index k
    const int c = idx >> 6, k = idx & 63;
    const int q = c >> 1, b = c & 1, pp = k >> 1, a = k & 1;
    const cpx<dd> j = Jm[pp * GP + q];
    const dd y = (a == b) ? j.x : (a == 0 ? j.y : -j.y);
    const float sc = vexp[pp];  // 2^e_p (exact scaling)
    float d[ND];
    oz_digits<ND>(__fmul_rn(y.hi, sc), __fmul_rn(y.lo, sc), Fcol[c], d);
    const uint32_t off = oz_elem(c, k, NN);
#pragma unroll
    for (int jj = 0; jj < ND; ++jj) Bp[size_t(jj) * NN * NN + off] = __float2bfloat16_rn(d[jj]);
  }
  const int r = tid & (MT - 1), g = tid >> 7;  // row of the tile; vectors 8g .. 8g + 7
  for (int i0 = 0; i0 < ell; i0 += MT) {
    const int i = i0 + r;
    cpx<dd> v[8];
    float mx = 0.f;
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int q = 8 * g + u;
      cpx<dd> x = czero<dd>();
      if (cols[q] >= 0 && i < ell) x = A[size_t(cols[q]) * ell + i];
      const float inv = 1.f / vexp[q];  // 2^-e_q
      x.x = dd(__fmul_rn(x.x.hi, inv), __fmul_rn(x.x.lo, inv));
      x.y = dd(__fmul_rn(x.y.hi, inv), __fmul_rn(x.y.lo, inv));
      v[u] = x;
      mx = fmaxf(mx, fmaxf(fabsf(x.x.hi), fabsf(x.y.hi)));
    }
    rmax[g * MT + r] = mx;
    __syncthreads();
    if (tid < MT)
      Erow[tid] = oz_exponent(fmaxf(fmaxf(rmax[tid], rmax[MT + tid]), fmaxf(rmax[2 * MT + tid], rmax[3 * MT + tid])));
    __syncthreads();
    const int E = Erow[r];
    for (int chunk = 0; chunk < 2; ++chunk) {
      if (chunk == 1) ok = wait_mma<dd, W>(sm) && ok;  // the planes of chunk 0 are free again
      if ((g >> 1) == chunk) {
#pragma unroll
        for (int u = 0; u < 8; ++u) {
#pragma unroll
          for (int a = 0; a < 2; ++a) {
            const dd x = a ? v[u].y : v[u].x;
            float d[ND];
            oz_digits<ND>(x.hi, x.lo, E, d);
            const uint32_t off = oz_elem(r, 16 * (g & 1) + 2 * u + a, KC);
#pragma unroll
            for (int jj = 0; jj < ND; ++jj) Ap[size_t(jj) * MT * KC + off] = __float2bfloat16_rn(d[jj]);
          }
        }
      }
      tc::fence_smem_to_async();
      __syncthreads();
      if (tid == 0) {
        tc::fence_after_sync();
        for (int lv = 0; lv < ND; ++lv) {
          for (int ja = 0; ja <= lv; ++ja) {
            const int jb = lv - ja;
#pragma unroll
            for (int ks = 0; ks < KC / 16; ++ks) {
              const uint64_t ad = tc::smem_desc(reinterpret_cast<char *>(Ap + size_t(ja) * MT * KC) + ks * 256, 128,
                                                KC * 16);
              const uint64_t bd = tc::smem_desc(
                  reinterpret_cast<char *>(Bp + size_t(jb) * NN * NN) + (chunk * (KC / 16) + ks) * 256, 128, NN * 16);
              tc::mma_bf16(sm.tmem + uint32_t(64 * lv), ad, bd, IDESC, (chunk > 0 || ja > 0 || ks > 0) ? 1u : 0u);
            }
          }
        }
        tc::mma_commit(sm.bar);
      }
    }
    ok = wait_mma<dd, W>(sm) && ok;
    tc::fence_after_sync();
    // epilogue: warp w reads rows 32 (w % 4) .. +31 and output columns 16 (w / 4) .. +15
    const int row = 32 * (warp & 3) + lane, cq = warp >> 2;
    dacc acc[16];
#pragma unroll
    for (int c = 0; c < 16; ++c) acc[c].hi = acc[c].lo = 0.f;
#pragma unroll 1
    for (int lv = 0; lv < ND; ++lv) {
      float t16[16];
      tc::tmem_ld16(sm.tmem + (uint32_t(32 * (warp & 3)) << 16) + uint32_t(64 * lv + 16 * cq), t16);
      const float wgt = pow2f(-7 * lv);
#pragma unroll
      for (int c = 0; c < 16; ++c) {
        float s, e;
        two_sum(acc[c].hi, __fmul_rn(t16[c], wgt), s, e);
        acc[c].hi = s;
        acc[c].lo = __fadd_rn(acc[c].lo, e);
      }
    }
    const int ii = i0 + row;
    if (ii < ell) {
#pragma unroll
      for (int qq = 0; qq < 8; ++qq) {
        const int q = 8 * cq + qq;
        if (cols[q] < 0) continue;
        const int sh = Erow[row] + Fcol[2 * q] - 14;
        const dd re = dd_norm(acc[2 * qq].hi, acc[2 * qq].lo), im = dd_norm(acc[2 * qq + 1].hi, acc[2 * qq + 1].lo);
        A[size_t(cols[q]) * ell + ii] = mkc<dd>(dd(scale2f(re.hi, sh), scale2f(re.lo, sh)),
                                              dd(scale2f(im.hi, sh), scale2f(im.lo, sh)));
      }
    }
    tc::fence_before_sync();
    __syncthreads();
  }
  return ok;
}

// A_b <- A_b J for a double-float block when J is within kappa of the
// identity (the finishing sweeps, after the guided ones: rotation angles of
// the order of the float threshold and below): A_b + A_b (J - I), the
// correction formed in float from the leading halves, which is accurate to
// about 2^-24 kappa of the vectors, and added to the double-float values
// exactly (TwoSum).  kappa <= 1e-6 keeps the correction's error below the
// double-float threshold of the convergence test.
template <int NT, int W>
__device__ void update_near_identity(cpx<dd> *__restrict__ A, int ell, const int *cols, const cpx<dd> *__restrict__ Jm,
                                     Smem<dd, W> &sm) {
  constexpr int TP = W + 1, GP = W + 1;
  cpx<float> *Ts = reinterpret_cast<cpx<float> *>(sm.Ts);       // 32 rows x W, hi parts
  cpx<float> *K = reinterpret_cast<cpx<float> *>(sm.Ts) + 32 * TP;  // W x W: J - I in float
  static_assert(sizeof(cpx<float>) * (32 * TP + W * GP) <= SmemLayout<dd, W>::ts_bytes, "fits Ts");
  for (int idx = threadIdx.x; idx < W * W; idx += NT) {
    const int pp = idx / W, q = idx % W;
    cpx<dd> j = Jm[pp * GP + q];
    if (pp == q) j.x = j.x - dd(1.f, 0.f);
    K[pp * GP + q] = mkc<float>(float(j.x), float(j.y));
  }
  constexpr int PER = (32 * W + NT - 1) / NT;
  for (int i0 = 0; i0 < ell; i0 += 32) {
    __syncthreads();
    for (int idx = threadIdx.x; idx < 32 * W; idx += NT) {
      const int r = idx & 31, q = idx >> 5;
      cpx<float> v = czero<float>();
      if (cols[q] >= 0 && i0 + r < ell) {
        const cpx<dd> x = A[size_t(cols[q]) * ell + i0 + r];
        v = mkc<float>(x.x.hi, x.y.hi);
      }
      Ts[r * TP + q] = v;
    }
    __syncthreads();
#pragma unroll
    for (int e = 0; e < PER; ++e) {
      const int o = threadIdx.x + e * NT;
      if (o < 32 * W) {
        const int q = o >> 5, r = o & 31;
        if (cols[q] >= 0 && i0 + r < ell) {
          cpx<float> c = czero<float>();
          for (int pp = 0; pp < W; ++pp) c = cfma(Ts[r * TP + pp], K[pp * GP + q], c);
          cpx<dd> &x = A[size_t(cols[q]) * ell + i0 + r];
          const cpx<dd> y = x;
          x = mkc<dd>(y.x + dd(c.x), y.y + dd(c.y));
        }
      }
    }
  }
  __syncthreads();
}

// -- resident path (float, ell <= RES_ROWS, W == 32) ---------------------
// Slots [s0, s0 + W/2) of Ab (Ab[r][s0 + p] = A[rc[s0 + p]][r]) from A, or
// back to A; eight independent accesses in flight per thread.  No barrier.
// Each thread moves a pair of adjacent slots (p, p + 1) of one row: two
// coalesced global accesses (consecutive lanes, consecutive rows) and one
// 16-byte shared access, which with the even row pitch is free of bank
// conflicts within each quarter warp.
template <typename T, int NT, int W>
__device__ void load_half_res(const cpx<T> *__restrict__ A, int ell, const int *rc, int s0, Smem<T, W> &sm) {
  constexpr int TP = SmemLayout<T, W>::AP, B = W / 2, UN = 4;
  static_assert(TP % 2 == 0 && sizeof(T) == 4, "16-byte pairs");
  const int tot = (B / 2) * ell;
  for (int base = threadIdx.x; base < tot; base += NT * UN) {
    cpx<T> v0[UN], v1[UN];
#pragma unroll
    for (int u = 0; u < UN; ++u) {
      const int idx = base + u * NT;
      const int pp = idx / ell, r = idx - pp * ell;
      const int c0 = idx < tot ? rc[s0 + 2 * pp] : -1, c1 = idx < tot ? rc[s0 + 2 * pp + 1] : -1;
      v0[u] = c0 >= 0 ? A[size_t(c0) * ell + r] : czero<T>();
      v1[u] = c1 >= 0 ? A[size_t(c1) * ell + r] : czero<T>();
    }
#pragma unroll
    for (int u = 0; u < UN; ++u) {
      const int idx = base + u * NT;
      const int pp = idx / ell, r = idx - pp * ell;
      if (idx < tot)
        *reinterpret_cast<float4 *>(sm.Ab + r * TP + s0 + 2 * pp) = make_float4(v0[u].x, v0[u].y, v1[u].x, v1[u].y);
    }
  }
}

template <typename T, int NT, int W>
__device__ void store_half_res(cpx<T> *__restrict__ A, int ell, const int *rc, int s0, const Smem<T, W> &sm) {
  constexpr int TP = SmemLayout<T, W>::AP, B = W / 2;
  static_assert(TP % 2 == 0 && sizeof(T) == 4, "16-byte pairs");
  for (int idx = threadIdx.x; idx < (B / 2) * ell; idx += NT) {
    const int pp = idx / ell, r = idx - pp * ell;
    const float4 v = *reinterpret_cast<const float4 *>(sm.Ab + r * TP + s0 + 2 * pp);
    const int c0 = rc[s0 + 2 * pp], c1 = rc[s0 + 2 * pp + 1];
    if (c0 >= 0) A[size_t(c0) * ell + r] = mkc<T>(v.x, v.y);
    if (c1 >= 0) A[size_t(c1) * ell + r] = mkc<T>(v.z, v.w);
  }
}

// G = Ab^H Ab, Hermitian: only the three 16 x 16 tiles G_II, G_IJ and G_JJ
// (I = slots 0-15, J = slots 16-31) are formed, G_JI = G_IJ^H is filled in
// after.  Warp w < 15 computes tile w % 3 over the rows r = w / 3 (mod 5) of
// Ab; lane = (tile column c = lane % 16, row half h = lane / 16), eight rows
// per lane read as four 16-byte broadcasts per half-warp.  The five partial
// sums (G itself, two compact tiles' worth in region 0 and one each in Ts and
// J, all free at this point) are added in a fixed order.
template <typename T, int NT, int W>
__device__ void gram_res(int ell, Smem<T, W> &sm) {
  static_assert(W == 32 && NT == 512, "resident Gram assumes W = 32, 16 warps");
  constexpr int TP = SmemLayout<T, W>::AP, GP = W + 1, RS = 8, KS = 5, NTILE = 3, TE = 256;
  static_assert(TP % 2 == 0, "16-byte aligned rows");
  static_assert(SmemLayout<T, W>::theta_bytes >= 2 * NTILE * TE * sizeof(cpx<T>), "two partials fit region 0");
  static_assert(SmemLayout<T, W>::ts_bytes >= NTILE * TE * sizeof(cpx<T>), "a partial fits Ts");
  static_assert(SmemLayout<T, W>::g_bytes >= NTILE * TE * sizeof(cpx<T>), "a partial fits J");
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int tile = warp % NTILE, ks = warp / NTILE;  // warp 15: ks = 5, idle
  const int row0 = tile == 2 ? 16 : 0, col0 = tile == 0 ? 0 : 16;
  const int c = lane & 15, h = lane >> 4;
  const int p0 = row0 + 8 * h, q = col0 + c;
  cpx<T> acc[RS];
#pragma unroll
  for (int i = 0; i < RS; ++i) acc[i] = czero<T>();
  if (ks < KS) {
    int r = ks;
    for (; r + KS < ell; r += 2 * KS) {
      const cpx<T> *ra = sm.Ab + r * TP, *rb = ra + KS * TP;
      const float4 *v0 = reinterpret_cast<const float4 *>(ra + p0), *v1 = reinterpret_cast<const float4 *>(rb + p0);
      const cpx<T> y0 = ra[q], y1 = rb[q];
#pragma unroll
      for (int i = 0; i < RS / 2; ++i) {
        const float4 a = v0[i], b = v1[i];
        acc[2 * i] = cjfma(mkc<T>(b.x, b.y), y1, cjfma(mkc<T>(a.x, a.y), y0, acc[2 * i]));
        acc[2 * i + 1] = cjfma(mkc<T>(b.z, b.w), y1, cjfma(mkc<T>(a.z, a.w), y0, acc[2 * i + 1]));
      }
    }
    if (r < ell) {
      const cpx<T> *ra = sm.Ab + r * TP;
      const cpx<T> y0 = ra[q];
#pragma unroll
      for (int i = 0; i < RS; ++i) acc[i] = cjfma(ra[p0 + i], y0, acc[i]);
    }
  }
  // partial ks: 0 -> G (pitch GP); 1, 2 -> region 0; 3 -> Ts; 4 -> J (compact, tile-major)
  cpx<T> *r0 = reinterpret_cast<cpx<T> *>(sm.r0);
  cpx<T> *P1 = r0, *P2 = r0 + NTILE * TE, *P3 = sm.Ts, *P4 = sm.J;
  if (ks == 0) {
#pragma unroll
    for (int i = 0; i < RS; ++i) sm.G[(p0 + i) * GP + q] = acc[i];
  } else if (ks < KS) {
    cpx<T> *dst = ks == 1 ? P1 : (ks == 2 ? P2 : (ks == 3 ? P3 : P4));
#pragma unroll
    for (int i = 0; i < RS; ++i) dst[tile * TE + (8 * h + i) * 16 + c] = acc[i];
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < NTILE * TE; idx += NT) {
    const int t = idx / TE, e = idx % TE, a = e / 16, b = e % 16;
    const int pp = (t == 2 ? 16 : 0) + a, qq = (t == 0 ? 0 : 16) + b;
    const int o = pp * GP + qq;
    sm.G[o] = cadd(cadd(sm.G[o], P1[idx]), cadd(cadd(P2[idx], P3[idx]), P4[idx]));
  }
  __syncthreads();
  // G_JI = G_IJ^H
  for (int idx = threadIdx.x; idx < TE; idx += NT) {
    const int a = idx / 16, b = idx % 16;
    const cpx<T> v = sm.G[b * GP + 16 + a];
    sm.G[(16 + a) * GP + b] = mkc<T>(v.x, -v.y);
  }
  __syncthreads();
}

// Ab <- Ab J in place (Ab resident, ell <= 4 * NT / 4 rows): thread owns
// 4 rows x 8 columns, all products formed before the barrier, then stored.
template <typename T, int NT, int W>
__device__ void update_res(int ell, const cpx<T> *__restrict__ Jm, Smem<T, W> &sm) {
  static_assert(W == 32 && NT % 4 == 0, "resident update layout");
  constexpr int TP = SmemLayout<T, W>::AP, RB = NT / 4;
  static_assert(SmemLayout<T, W>::RES_ROWS <= 4 * RB, "one pass covers every resident row");
  const int qb = threadIdx.x / RB, rb = threadIdx.x % RB;
  const int q0 = qb * 8;
  cpx<T> acc[4][8];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[i][j] = czero<T>();
  static_assert(TP % 2 == 0 && sizeof(T) == 4, "16-byte pairs");
  for (int p = 0; p < W; p += 2) {
    // slots p, p + 1 of each of the thread's rows in one 16-byte read
    float4 a2[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int r = rb + i * RB;
      a2[i] = r < ell ? *reinterpret_cast<const float4 *>(sm.Ab + r * TP + p) : make_float4(0.f, 0.f, 0.f, 0.f);
    }
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      cpx<T> jr[8];
#pragma unroll
      for (int j = 0; j < 8; ++j) jr[j] = Jm[(p + h) * (W + 1) + q0 + j];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const cpx<T> a = h ? mkc<T>(a2[i].z, a2[i].w) : mkc<T>(a2[i].x, a2[i].y);
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[i][j] = cfma(a, jr[j], acc[i][j]);
      }
    }
  }
  __syncthreads();
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int r = rb + i * RB;
    if (r < ell) {
      float4 *dst = reinterpret_cast<float4 *>(sm.Ab + r * TP + q0);
#pragma unroll
      for (int j = 0; j < 4; ++j)
        dst[j] = make_float4(acc[i][2 * j].x, acc[i][2 * j].y, acc[i][2 * j + 1].x, acc[i][2 * j + 1].y);
    }
  }
  __syncthreads();
}

// Rotation of the Hermitian 2x2 [[a, g], [conj g, b]] that zeroes g
// (Rutishauser's formulas: t = sign(zeta) / (|zeta| + sqrt(1 + zeta^2)),
// zeta = (b - a) / 2|g|, c = 1/sqrt(1 + t^2), s = t c, e = conj(g)/|g|), or
// false when the pair is below the threshold |g| > tol sqrt(a b) or either
// diagonal is rounding noise.  float: the reciprocal square root and the
// division run on the approximate special-function path (a few ulp); c and
// s come from the same t, so the rotation stays orthogonal to rounding and
// an error in t only leaves a residual far below the threshold.
template <typename T>
__device__ __forceinline__ bool jacobi_rotation(T a, T b, cpx<T> g, T tol, T tiny2, T &c, T &sn, cpx<T> &e) {
  const T ag = sqrt(cabs2(g));
  if (!(a > tiny2 && b > tiny2 && ag > tol * sqrt(a) * sqrt(b))) return false;
  const T zeta = (b - a) / (T(2) * ag);
  T t_ = T(1) / (fabs(zeta) + sqrt(T(1) + zeta * zeta));
  if (zeta < T(0)) t_ = -t_;
  c = T(1) / sqrt(T(1) + t_ * t_);
  sn = t_ * c;
  e = mkc<T>(g.x / ag, -g.y / ag);  // e^{-i phi}, g = |g| e^{i phi}
  return true;
}

template <>
__device__ __forceinline__ bool jacobi_rotation<float>(float a, float b, cpx<float> g, float tol, float tiny2,
                                                       float &c, float &sn, cpx<float> &e) {
  const float g2 = fmaf(g.x, g.x, g.y * g.y);
  if (!(a > tiny2 && b > tiny2 && g2 > (tol * tol) * (a * b))) return false;
  const float rg = rsqrtf(g2);  // 1 / |g|
  const float zeta = (b - a) * (0.5f * rg);
  const float z1 = fmaf(zeta, zeta, 1.f);
  const float t_ = copysignf(__fdividef(1.f, fabsf(zeta) + z1 * rsqrtf(z1)), zeta);
  c = rsqrtf(fmaf(t_, t_, 1.f));
  sn = t_ * c;
  e = mkc<float>(g.x * rg, -g.y * rg);
  return true;
}

// Whether the pair (a, b, g) of a Gram matrix needs a rotation: both
// diagonals above the noise level and |g| > tol sqrt(a b).
template <typename T>
__device__ __forceinline__ bool pair_active(T a, T b, cpx<T> g, T tol, T tiny2) {
  const T ag = sqrt(cabs2(g));
  return a > tiny2 && b > tiny2 && ag > tol * sqrt(a) * sqrt(b);
}

// |g| of a dd complex value without squaring it (the square of a small Gram
// entry would leave float32's range): the larger part times
// sqrt(1 + (smaller / larger)^2); also the unit phase g / |g|.
__device__ __forceinline__ dd dd_cabs(cpx<dd> g, cpx<dd> *phase) {
  const dd gx = fabs(g.x), gy = fabs(g.y);
  const bool xl = !(gx < gy);
  const dd mx = xl ? gx : gy;
  if (!(mx.hi > 0.f)) {
    if (phase) *phase = mkc<dd>(dd(1.f, 0.f), dd(0.f, 0.f));
    return dd(0.f, 0.f);
  }
  const dd ux = g.x / mx, uy = g.y / mx;  // components of g / max(|gx|, |gy|)
  const dd r = sqrt(ux * ux + uy * uy);  // in [1, sqrt 2]
  if (phase) *phase = mkc<dd>(ux / r, -(uy / r));
  return mx * r;
}

// |g| / sqrt(a b) of a double-float Gram pair, divided step by step to stay
// in range; 0 when either diagonal is at the noise level.
__device__ __forceinline__ dd pair_ratio(dd a, dd b, cpx<dd> g, dd tiny2) {
  if (!(a > tiny2 && b > tiny2)) return dd(0.f, 0.f);
  return (dd_cabs(g, nullptr) / sqrt(a)) / sqrt(b);
}

template <>
__device__ __forceinline__ bool pair_active<dd>(dd a, dd b, cpx<dd> g, dd tol, dd tiny2) {
  return pair_ratio(a, b, g, tiny2) > tol;
}

// The double-float rotation: the formulas of the generic version, with |g|
// and the phase from dd_cabs and t = 1 / (2 |zeta|) once zeta^2 would
// overflow float32 (|zeta| > 1e15, where sqrt(1 + zeta^2) = |zeta| to the
// working precision).
template <>
__device__ __forceinline__ bool jacobi_rotation<dd>(dd a, dd b, cpx<dd> g, dd tol, dd tiny2, dd &c, dd &sn,
                                                    cpx<dd> &e) {
  if (!(a > tiny2 && b > tiny2)) return false;
  const dd ag = dd_cabs(g, &e);
  if (!((ag / sqrt(a)) / sqrt(b) > tol)) return false;
  const dd zeta = (b - a) / (dd(2.f) * ag);
  const dd az = fabs(zeta);
  dd t_ = az.hi > 1e15f ? dd(0.5f) / az : dd(1.f) / (az + sqrt(dd(1.f) + az * az));
  if (zeta.hi < 0.f) t_ = -t_;
  c = dd(1.f) / sqrt(dd(1.f) + t_ * t_);
  sn = t_ * c;
  return true;
}

// One cyclic sweep of two-sided Jacobi on the Hermitian W x W matrix in
// sm.G (row pitch W + 1) with round-robin ordering, accumulating J (same
// pitch).  Warp t owns rotation pair t of every round: all its lanes compute
// the pair's rotation from G, apply R^H to rows p, q of G (lane = column),
// then, after a barrier, R to columns p, q of G and J (lane = row).  Pairs
// of one round are disjoint, so each element has one writer per phase.
template <typename T, int NT, int W>
__device__ const cpx<T> *jacobi_gram(Smem<T, W> &sm, const int *cols, T tol, T tiny2, int mode, int inner = 1) {
  constexpr int H = W / 2, GP = W + 1;
  static_assert(W == 32 && NT / 32 == H, "one warp per rotation pair");
  cpx<T> *G = sm.G, *J = sm.J;
  const int lane = threadIdx.x & 31, t = threadIdx.x >> 5;
  // J = I (G was written before the caller's barrier; J is first read after
  // the barrier of round 0)
  for (int idx = threadIdx.x; idx < W * W; idx += NT) {
    int p = idx / W, q = idx % W;
    J[p * GP + q] = (p == q) ? mkc<T>(T(1), T(0)) : czero<T>();
  }
  // mode 0: all pairs of the W vectors (W-1 rounds); mode 1: only pairs
  // across the two halves (H rounds); mode 2: only pairs within each half
  // (H-1 rounds).  Every round rotates H disjoint pairs.
  const int rounds = mode == 0 ? W - 1 : (mode == 1 ? H : H - 1);
  for (int r = 0; r < rounds * inner; ++r) {
    int p, q;
    if (mode == 0) {
      rr_pair<W>(r, t, p, q);
    } else if (mode == 1) {
      p = t;
      q = H + (t + r) % H;
    } else {
      const int h = t / (H / 2), tt = t % (H / 2);
      rr_pair<H>(r, tt, p, q);
      p += h * H;
      q += h * H;
    }
    // R on (p, q): column p = (c, -s e), column q = (s, c e)
    T c = T(1), sn = T(0);
    cpx<T> e = mkc<T>(T(1), T(0));
    // an empty slot (cols < 0) holds a zero vector, so its Gram diagonal is 0
    // <= tiny2 and jacobi_rotation declines the pair without reading cols
    const bool rot = jacobi_rotation<T>(G[p * GP + p].x, G[q * GP + q].x, G[p * GP + q], tol, tiny2, c, sn, e);
    __syncwarp();  // every lane has read the pivot entries before row p, q change
    if (rot) {
      // rows: G[p][j] <- c G[p][j] - s conj(e) G[q][j];  G[q][j] <- s G[p][j] + c conj(e) G[q][j]
      const cpx<T> gp = G[p * GP + lane], gq = G[q * GP + lane];
      const cpx<T> egq = cmul(mkc<T>(e.x, -e.y), gq);
      G[p * GP + lane] = mkc<T>(c * gp.x - sn * egq.x, c * gp.y - sn * egq.y);
      G[q * GP + lane] = mkc<T>(sn * gp.x + c * egq.x, sn * gp.y + c * egq.y);
    }
    __syncthreads();
    if (rot) {
      // columns: X[i][p] <- c X[i][p] - s e X[i][q];  X[i][q] <- s X[i][p] + c e X[i][q]
      const int i = lane;
      const cpx<T> gp = G[i * GP + p], gq = cmul(e, G[i * GP + q]);
      G[i * GP + p] = mkc<T>(c * gp.x - sn * gq.x, c * gp.y - sn * gq.y);
      G[i * GP + q] = mkc<T>(sn * gp.x + c * gq.x, sn * gp.y + c * gq.y);
      const cpx<T> jp = J[i * GP + p], jq = cmul(e, J[i * GP + q]);
      J[i * GP + p] = mkc<T>(c * jp.x - sn * jq.x, c * jp.y - sn * jq.y);
      J[i * GP + q] = mkc<T>(sn * jp.x + c * jq.x, sn * jp.y + c * jq.y);
    }
    __syncthreads();
  }
  return J;
}

// The inner sweep of a guided step (jacobi_svd<dd>): the rotations are
// chosen on the float Gram in sm.G's area exactly as jacobi_gram chooses
// them, but each is rebuilt in double-float as an exactly unitary rotation
// -- c = 1 / sqrt(1 + t^2), s = t c from the float tangent t = s / c, the
// phase e normalised to modulus 1 -- and only those rebuilt rotations are
// accumulated into J (double-float).  The angles are float accurate, which
// is all an early sweep needs; J stays unitary to the double-float rounding,
// so applying it to the double-float vectors changes no singular value
// beyond that rounding.
template <int NT, int W>
__device__ const cpx<dd> *jacobi_gram_guided(Smem<dd, W> &sm, float tol, float tiny2, int mode, int inner) {
  constexpr int H = W / 2, GP = W + 1;
  static_assert(W == 32 && NT / 32 == H, "one warp per rotation pair");
  cpx<float> *G = reinterpret_cast<cpx<float> *>(sm.G);
  cpx<dd> *J = sm.J;
  const int lane = threadIdx.x & 31, t = threadIdx.x >> 5;
  for (int idx = threadIdx.x; idx < W * W; idx += NT) {
    const int p = idx / W, q = idx % W;
    J[p * GP + q] = (p == q) ? mkc<dd>(dd(1.f, 0.f), dd(0.f, 0.f)) : czero<dd>();
  }
  const int rounds = mode == 0 ? W - 1 : (mode == 1 ? H : H - 1);
  for (int r = 0; r < rounds * inner; ++r) {
    int p, q;
    if (mode == 0) {
      rr_pair<W>(r, t, p, q);
    } else if (mode == 1) {
      p = t;
      q = H + (t + r) % H;
    } else {
      const int h = t / (H / 2), tt = t % (H / 2);
      rr_pair<H>(r, tt, p, q);
      p += h * H;
      q += h * H;
    }
    float c = 1.f, sn = 0.f;
    cpx<float> e = mkc<float>(1.f, 0.f);
    const bool rot = jacobi_rotation<float>(G[p * GP + p].x, G[q * GP + q].x, G[p * GP + q], tol, tiny2, c, sn, e);
    __syncwarp();
    if (rot) {
      const cpx<float> gp = G[p * GP + lane], gq = G[q * GP + lane];
      const cpx<float> egq = cmul(mkc<float>(e.x, -e.y), gq);
      G[p * GP + lane] = mkc<float>(c * gp.x - sn * egq.x, c * gp.y - sn * egq.y);
      G[q * GP + lane] = mkc<float>(sn * gp.x + c * egq.x, sn * gp.y + c * egq.y);
    }
    __syncthreads();
    if (rot) {
      const int i = lane;
      const cpx<float> gp = G[i * GP + p], gq = cmul(e, G[i * GP + q]);
      G[i * GP + p] = mkc<float>(c * gp.x - sn * gq.x, c * gp.y - sn * gq.y);
      G[i * GP + q] = mkc<float>(sn * gp.x + c * gq.x, sn * gp.y + c * gq.y);
      // the same rotation, exactly unitary in double-float
      const dd td = dd(sn) / dd(c);
      const dd cd = dd(1.f) / sqrt(dd(1.f) + td * td), sd = td * cd;
      const dd ex = dd(e.x), ey = dd(e.y);
      const dd er = sqrt(ex * ex + ey * ey);
      const cpx<dd> ed = mkc<dd>(ex / er, ey / er);
      const cpx<dd> jp = J[i * GP + p], jq = cmul(ed, J[i * GP + q]);
      J[i * GP + p] = mkc<dd>(cd * jp.x - sd * jq.x, cd * jp.y - sd * jq.y);
      J[i * GP + q] = mkc<dd>(sd * jp.x + cd * jq.x, sd * jp.y + cd * jq.y);
    }
    __syncthreads();
  }
  return J;
}

template <typename T, int NT, int W>
__device__ void bitonic_desc(double *key, int *idx, int P);

template <typename T, int NT, int W>
__device__ int jacobi_svd(cpx<T> *__restrict__ A, int ell, int c, int max_sweeps, Smem<T, W> &sm,
                          long long *cyc, double *__restrict__ nrm, int *__restrict__ ord, int scheme) {
  using L = SmemLayout<T, W>;
  constexpr int B = W / 2;
  const bool resident = (L::RES_ROWS > 0) && ell <= L::RES_ROWS;
  // Rounding noise of a computed Gram entry is about sqrt(ell) eps |a_p||a_q|;
  // the threshold sits a factor 4 above it so that converged pairs are not
  // rotated again on noise alone.
  const T tol = T(4) * sqrt(T(ell)) * Eps<T>::v;
  // Double-float: the sweeps start guided (float Gram of the hi parts, float
  // rotation angles, double-float rotations and update) until a sweep finds
  // no pair above the float threshold; the last sweeps run in double-float.
  //
  // Cyclic Jacobi converges quadratically near the end: a sweep whose pairs
  // all had |g| <= r sqrt(a b) before their rotations leaves pairs of order
  // r^2 / (relative gap).  So a guided sweep with every pair below
  // kGuidedDone (1e-4: the next guided sweep would find ~1e-8 / gap, under
  // the float threshold ~5e-6) hands over to double-float at once instead of
  // running one more float Gram only to find nothing, and a double-float sweep with
  // every pair below kFinishDone (1e-9: what is left is ~1e-18 / gap, under
  // the double-float threshold tol ~6e-13 for relative gaps down to 1e-5)
  // is the last one, instead of a further Gram pass that only confirms it.
  constexpr bool kDD = std::is_same<T, dd>::value;
  bool guided = kDD;
  const float tol_f = 4.f * sqrtf(float(ell)) * Eps<float>::v;
  constexpr float kGuidedDone = 1e-4f, kFinishDone = 1e-9f;
  // Columns with |a|^2 <= eps^2 ||A||_F^2 are rounding noise: rotating them
  // changes nothing above rounding and their relative off-diagonals never
  // settle, so they are neither rotated nor counted for convergence.
  double fro = 0.0;
  for (size_t idx = threadIdx.x; idx < size_t(ell) * c; idx += NT) {
    cpx<T> x = A[idx];
    fro += double(x.x * x.x + x.y * x.y);
  }
  fro = block_sum<NT>(fro, sm.red);
  const T tiny2 = T(fro * sweep_floor<T>(ell) * sweep_floor<T>(ell));
  const float tiny2_f = float(fro * double(Eps<float>::v) * double(Eps<float>::v));
  const int nblk = (c + B - 1) / B;
  int *cols = sm.ired + 128;  // W ints (ired[0..128) is reduction scratch)
  // Column norms^2, kept current from the rotated Gram diagonals; each sweep
  // visits the columns in decreasing-norm order (de Rijk's ordering), which
  // shortens the one-sided Jacobi iteration.
  if (nblk > 2) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int j = warp; j < c; j += NT / 32) {
      T part = T(0);
      for (int i = lane; i < ell; i += 32) part += cabs2(A[size_t(j) * ell + i]);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) part += shfl_xor(part, o);
      if (lane == 0) nrm[j] = double(part);
    }
    __syncthreads();
  }
  // Resident path: Ab keeps the two half-blocks of the last step (block ids
  // resI, resJ, columns rcols) across steps; a half is written back to A
  // only when another block replaces it, before the sweep's re-ordering, and
  // on return.  Consecutive steps (I, J), (I, J+1) then move one half only.
  int *rcols = sm.ired + 128 + W;
  int resI = -1, resJ = -1;
  bool dirtyI = false, dirtyJ = false;
  auto flush = [&]() {
    if constexpr (L::RES_ROWS > 0) {
      if (resident) {
        if (dirtyI) store_half_res<T, NT, W>(A, ell, rcols, 0, sm);
        if (dirtyJ) store_half_res<T, NT, W>(A, ell, rcols, B, sm);
        __syncthreads();
      }
    }
    dirtyI = dirtyJ = false;
    resI = resJ = -1;
  };
  for (int sweep = 0; sweep < max_sweeps; ++sweep) {
    int rotated = 0;
    int far = 0;  // (double-float) some pair of this sweep above kGuidedDone / kFinishDone
    if (nblk > 2) {
      flush();  // the re-ordering changes which columns a block id names
      int P = 1;
      while (P < c) P <<= 1;
      double *key = reinterpret_cast<double *>(sm.r0);
      int *kidx = reinterpret_cast<int *>(key + P);
      for (int j = threadIdx.x; j < P; j += NT) {
        key[j] = j < c ? nrm[j] : -1.0;
        kidx[j] = j;
      }
      __syncthreads();
      bitonic_desc<T, NT, W>(key, kidx, P);
      for (int j = threadIdx.x; j < c; j += NT) ord[j] = kidx[j];
      __syncthreads();
    }
    // Steps of one sweep: nblk <= 2 -> one step over all c vectors (every
    // pair).  Otherwise every pair is visited once: ceil(nblk/2) steps over
    // block pairs (2b, 2b+1) rotating only pairs inside each block, then one
    // step per block pair I < J rotating only pairs across the two blocks.
    // Slots [0, B) hold block I, [B, W) block J; cols[t] = -1 marks an empty slot.
    // scheme 0: every step rotates all pairs of its block pair; 1: within-block
    // steps, then cross-block steps; 2: as 0 with two inner sweeps per step in
    // the first two outer sweeps (fewer outer sweeps for far-from-orthogonal
    // starts, such as a gate's theta)
    const int pscheme = scheme == 1 ? 1 : 0;  // scheme 3: as 2 over the first three sweeps
    const int inner = (scheme == 2 && sweep < 2) || (scheme == 3 && sweep < 3) ? 2 : 1;
    const int ndiag = (nblk <= 2 || pscheme == 0) ? 0 : (nblk + 1) / 2;
    const int nsteps = (nblk <= 2) ? 1 : ndiag + nblk * (nblk - 1) / 2;
    int I = 0, Jb = 1;
    for (int st = 0; st < nsteps; ++st) {
      int mode, bi, bj;
      if (nblk <= 2) {
        mode = 0;
        bi = 0;
        bj = 1;
      } else if (st < ndiag) {
        mode = 2;
        bi = 2 * st;
        bj = (2 * st + 1 < nblk) ? 2 * st + 1 : -1;
      } else {
        mode = pscheme == 0 ? 0 : 1;
        bi = I;
        bj = Jb;
        if (++Jb >= nblk) {
          ++I;
          Jb = I + 1;
        }
      }
      const int wi = min(B, c - bi * B), wj = bj >= 0 ? max(0, min(B, c - bj * B)) : 0;
      if (threadIdx.x < W) {
        const int t = threadIdx.x;
        int col = -1;
        if (t < B) {
          if (t < wi) col = (nblk > 2) ? ord[bi * B + t] : bi * B + t;
        } else if (t - B < wj) {
          col = (nblk > 2) ? ord[bj * B + (t - B)] : bj * B + (t - B);
        }
        cols[t] = col;
      }
      // The next cross-block step (I, Jb) keeps block I resident and loads
      // block Jb: start moving Jb's columns (contiguous, ell values each)
      // towards L2 now, one 128-byte line per thread, so that the load at the
      // next step does not wait on HBM.
      if constexpr (L::RES_ROWS > 0) {
        if (resident && nblk > 2 && st >= ndiag && st + 1 < nsteps && Jb < nblk) {
          const int wn = min(B, c - Jb * B);
          const int lines = (ell * int(sizeof(cpx<T>)) + 127) / 128;
          for (int idx = threadIdx.x; idx < wn * lines; idx += NT) {
            const int t = idx / lines, ln = idx - t * lines;
            const char *ptr = reinterpret_cast<const char *>(A + size_t(ord[Jb * B + t]) * ell) + size_t(ln) * 128;
            asm volatile("prefetch.global.L2 [%0];" ::"l"(ptr));
          }
        }
      }
      __syncthreads();
      long long t0 = clock64();
      if constexpr (L::RES_ROWS > 0) {
        if (resident) {
          const bool keepI = bi == resI, keepJ = bj >= 0 && bj == resJ;
          if (!keepI && dirtyI) store_half_res<T, NT, W>(A, ell, rcols, 0, sm);
          if (!keepJ && dirtyJ) store_half_res<T, NT, W>(A, ell, rcols, B, sm);
          __syncthreads();
          if (!keepI) load_half_res<T, NT, W>(A, ell, cols, 0, sm);
          if (!keepJ) load_half_res<T, NT, W>(A, ell, cols, B, sm);
          if (threadIdx.x < W) rcols[threadIdx.x] = cols[threadIdx.x];
          __syncthreads();
          dirtyI = dirtyI && keepI;
          dirtyJ = dirtyJ && keepJ;
          resI = bi;
          resJ = bj;
          gram_res<T, NT, W>(ell, sm);
        } else {
          gram_stream<T, NT, W>(A, ell, cols, sm);
        }
      } else {
        if constexpr (kDD) {
          if (guided)
            gram_stream_hi<NT, W>(A, ell, cols, sm);
          else
            gram_stream_herm<NT, W>(A, ell, cols, sm);
        } else {
          gram_stream<T, NT, W>(A, ell, cols, sm);
        }
      }
      // Pairs above the threshold, split into pairs inside a half-block and
      // pairs across the two halves.  A step whose within-half pairs are all
      // converged rotates only the cross pairs (H rounds instead of W-1), and
      // vice versa; a sweep still ends only when no pair of any step needs a
      // rotation, so convergence is decided on every pair as before.
      int needW = 0, needC = 0, farS = 0;
      for (int idx = threadIdx.x; idx < W * W; idx += NT) {
        int p = idx / W, q = idx % W;
        if (p < q && cols[p] >= 0 && cols[q] >= 0) {
          const bool cross = (p < B) != (q < B);
          if (mode == 1 && !cross) continue;
          if (mode == 2 && cross) continue;
          bool act;
          if (kDD && guided) {
            const cpx<float> *Gf = reinterpret_cast<const cpx<float> *>(sm.G);
            const float a = Gf[p * (W + 1) + p].x, b = Gf[q * (W + 1) + q].x;
            act = pair_active<float>(a, b, Gf[p * (W + 1) + q], tol_f, tiny2_f);
            farS |= int(pair_active<float>(a, b, Gf[p * (W + 1) + q], kGuidedDone, tiny2_f));
          } else {
            if constexpr (kDD) {
              const dd r = pair_ratio(sm.G[p * (W + 1) + p].x, sm.G[q * (W + 1) + q].x, sm.G[p * (W + 1) + q], tiny2);
              act = r > tol;
              farS |= int(r.hi > kFinishDone);
            } else {
              act = pair_active<T>(sm.G[p * (W + 1) + p].x, sm.G[q * (W + 1) + q].x, sm.G[p * (W + 1) + q], tol,
                                   tiny2);
            }
          }
          if (act) {
            if (cross)
              needC = 1;
            else
              needW = 1;
          }
        }
      }
      needW = __syncthreads_or(needW);
      needC = __syncthreads_or(needC);
      if constexpr (kDD) far |= __syncthreads_or(farS);
      const int need = needW | needC;
      if (mode == 0 && !(needW && needC)) mode = needC ? 1 : 2;
      long long t1 = clock64();
      cyc[0] += t1 - t0;
      cyc[3] += 1;
      if (need) {
        rotated = 1;
        // the vectors' squared norms before this step's rotations (scales of
        // the tensor-core update)
        float *gdiag = reinterpret_cast<float *>(sm.red);
        if (kDD && threadIdx.x < W) {
          if (guided)
            gdiag[threadIdx.x] = reinterpret_cast<const cpx<float> *>(sm.G)[threadIdx.x * (W + 2)].x;
          else
            gdiag[threadIdx.x] = float(double(sm.G[threadIdx.x * (W + 2)].x));
        }
        const cpx<T> *Jm;
        if constexpr (kDD) {
          Jm = guided ? jacobi_gram_guided<NT, W>(sm, tol_f, tiny2_f, mode, inner)
                      : jacobi_gram<T, NT, W>(sm, cols, tol, tiny2, mode, inner);
        } else {
          Jm = jacobi_gram<T, NT, W>(sm, cols, tol, tiny2, mode, inner);
        }
        long long t2 = clock64();
        cyc[1] += t2 - t1;
        t1 = t2;
        if constexpr (L::RES_ROWS > 0) {
          if (resident) {
            update_res<T, NT, W>(ell, Jm, sm);
            dirtyI = dirtyJ = true;
          } else {
            update_stream<T, NT, W>(A, ell, ell, cols, Jm, sm);
          }
        } else {
          if constexpr (kDD) {
            // finishing sweeps: how far J is from the identity (largest entry of J - I)
            int near_id = 0;
            if (!guided) {
              float kmax = 0.f;
              for (int idx = threadIdx.x; idx < W * W; idx += NT) {
                const int pp = idx / W, q = idx % W;
                cpx<dd> j = Jm[pp * (W + 1) + q];
                if (pp == q) j.x = j.x - dd(1.f, 0.f);
                kmax = fmaxf(kmax, fmaxf(fabsf(j.x.hi), fabsf(j.y.hi)));
              }
              near_id = __syncthreads_and(kmax <= 1e-6f);
            }
            // guided sweeps: the tensor-core update; finishing sweeps: the
            // float correction when J is near the identity, else the exact
            // double-float update (the finishing sweeps decide convergence at the
            // double-float threshold, so they take no other rounding)
            if (near_id)
              update_near_identity<NT, W>(A, ell, cols, Jm, sm);
            else if (sm.tc && guided)
              update_ozaki<NT, W>(A, ell, cols, Jm, gdiag, sm);
            else
              update_stream<T, NT, W>(A, ell, ell, cols, Jm, sm);
          } else {
            update_stream<T, NT, W>(A, ell, ell, cols, Jm, sm);
          }
        }
        if (nblk > 2 && threadIdx.x < W && cols[threadIdx.x] >= 0) {
          if (kDD && guided)
            nrm[cols[threadIdx.x]] = double(reinterpret_cast<const cpx<float> *>(sm.G)[threadIdx.x * (W + 2)].x);
          else
            nrm[cols[threadIdx.x]] = double(sm.G[threadIdx.x * (W + 2)].x);
        }
        cyc[2] += clock64() - t1;
      }
    }
    if (!rotated || (kDD && !far)) {
      if (guided) {  // float-converged: the remaining sweeps in double-float
        guided = false;
        continue;
      }
      flush();
      return sweep + 1;
    }
  }
  flush();
  return -1;
}

// =======================================================================
// Phase 3: singular values, sort, process_svd (mps.rs:236-293), Gamma
// rebuild (mps.rs:856-877 / 1357-1382), local_renormalize (1206-1209).
// =======================================================================
template <typename T, int NT, int W>
__device__ void bitonic_desc(double *key, int *idx, int P) {
  // order: key descending, index ascending on ties
  for (int k = 2; k <= P; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int t = threadIdx.x; t < P; t += NT) {
        int l = t ^ j;
        if (l > t) {
          bool up = ((t & k) == 0);
          double ka = key[t], kb = key[l];
          int ia = idx[t], ib = idx[l];
          bool a_first = (ka > kb) || (ka == kb && ia < ib);
          bool swap = up ? !a_first : a_first;
          if (swap) {
            key[t] = kb;
            key[l] = ka;
            idx[t] = ib;
            idx[l] = ia;
          }
        }
      }
      __syncthreads();
    }
  }
}

// C[x][y] = sum_k P(x,k) Q(y,k) over 64x64 output tiles (8 per thread),
// K staged through shared memory in chunks of 16; E(x, y, value) stores.
template <typename T, int NT, int W, class FP, class FQ, class FE>
__device__ void gemm_nt(int M, int N, int K, FP P, FQ Q, FE E, Smem<T, W> &sm) {
  using L = SmemLayout<T, W>;
  constexpr int GK = L::GK, GT = L::GT, PITCH = GT + 1;
  static_assert(NT == 512, "gemm_nt thread layout");
  cpx<T> *Ps = reinterpret_cast<cpx<T> *>(sm.r0);  // [GK][GT+1]
  cpx<T> *Qs = Ps + GK * PITCH;                    // [GK][GT+1]
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;  // 16 x 32
  for (int x0 = 0; x0 < M; x0 += GT) {
    for (int y0 = 0; y0 < N; y0 += GT) {
      typename CAcc<T>::type acc[4][2];
#pragma unroll
      for (int i = 0; i < 4; ++i) acc[i][0] = acc[i][1] = acc_zero<T>();
      for (int k0 = 0; k0 < K; k0 += GK) {
        __syncthreads();
        for (int idx = threadIdx.x; idx < GK * GT; idx += NT) {
          int kk = idx % GK, xx = idx / GK;
          int gx = x0 + xx, gk = k0 + kk;
          Ps[kk * PITCH + xx] = (gx < M && gk < K) ? P(gx, gk) : czero<T>();
          int gy = y0 + xx;
          Qs[kk * PITCH + xx] = (gy < N && gk < K) ? Q(gy, gk) : czero<T>();
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < GK; ++kk) {
          cpx<T> pv[4], qv[2];
#pragma unroll
          for (int i = 0; i < 4; ++i) pv[i] = Ps[kk * PITCH + tx * 4 + i];
#pragma unroll
          for (int j = 0; j < 2; ++j) qv[j] = Qs[kk * PITCH + ty * 2 + j];
#pragma unroll
          for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 2; ++j) acc_fma<T>(acc[i][j], pv[i], qv[j]);
        }
      }
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j) {
          int x = x0 + tx * 4 + i, y = y0 + ty * 2 + j;
          if (x < M && y < N) E(x, y, acc_fin<T>(acc[i][j]));
        }
    }
  }
  __syncthreads();
}

// C[x][y] = sum_k P(x, k) Q(y, k) (complex) on the tensor cores: the real view
// of P (interleaved re/im along K) times the 2x2 real embedding of Q, in
// 128 x 256 tcgen05 kind::tf32 tiles with 3xTF32 splitting, as in
// build_theta_tc; output columns of a tile ordered (y, re/im); E(x, y, v)
// stores.  Staging tiles in the resident Jacobi block's shared memory, which
// is idle outside the Jacobi.
template <int NT, int W, class FP, class FQ, class FE>
__device__ bool gemm_nt_tc(int M, int N, int K, FP P, FQ Q, FE E, Smem<float, W> &sm) {
  constexpr int MT = 128, NTL = 256, KC = 32, YT = NTL / 2;
  constexpr uint32_t IDESC = tc::idesc_tf32(MT, NTL);
  constexpr uint32_t LBO = 128, SBO = KC * 32;
  float *Ahi = reinterpret_cast<float *>(sm.Ab), *Alo = Ahi + MT * KC, *Bhi = Alo + MT * KC, *Blo = Bhi + NTL * KC;
  const int K2 = 2 * K;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  bool ok = true;
  for (int i0 = 0; i0 < M; i0 += MT) {
    for (int y0 = 0; y0 < N; y0 += YT) {
      int chunk = 0;
      for (int k0 = 0; k0 < K2; k0 += KC, ++chunk) {
        if (chunk > 0) ok = wait_mma<float, W>(sm) && ok;
        for (int idx = tid; idx < MT * KC; idx += NT) {
          const int core = idx >> 5, within = idx & 31;
          const int r = (core / (KC / 4)) * 8 + (within >> 2), kr = (core % (KC / 4)) * 4 + (within & 3);
          const int x = i0 + r, kk = k0 + kr;
          float v = 0.f;
          if (x < M && kk < K2) {
            const cpx<float> a = P(x, kk >> 1);
            v = (kk & 1) ? a.y : a.x;
          }
          float hi, lo;
          tc::split_tf32(v, hi, lo);
          Ahi[idx] = hi;
          Alo[idx] = lo;
        }
        for (int idx = tid; idx < NTL * KC; idx += NT) {
          const int core = idx >> 5, within = idx & 31;
          const int nl = (core / (KC / 4)) * 8 + (within >> 2), kr = (core % (KC / 4)) * 4 + (within & 3);
          const int kk = k0 + kr, a = kk & 1, b = nl & 1, y = y0 + (nl >> 1);
          float v = 0.f;
          if (y < N && kk < K2) {
            const cpx<float> q = Q(y, kk >> 1);
            v = (a == b) ? q.x : (a == 0 ? q.y : -q.y);  // [[Qr, Qi], [-Qi, Qr]]
          }
          float hi, lo;
          tc::split_tf32(v, hi, lo);
          Bhi[idx] = hi;
          Blo[idx] = lo;
        }
        tc::fence_smem_to_async();
        __syncthreads();
        if (tid == 0) {
          tc::fence_after_sync();
#pragma unroll
          for (int st = 0; st < KC / 8; ++st) {
            const uint32_t off = uint32_t(st) * 2 * LBO;
            const uint64_t ah = tc::smem_desc(reinterpret_cast<char *>(Ahi) + off, LBO, SBO);
            const uint64_t al = tc::smem_desc(reinterpret_cast<char *>(Alo) + off, LBO, SBO);
            const uint64_t bh = tc::smem_desc(reinterpret_cast<char *>(Bhi) + off, LBO, SBO);
            const uint64_t bl = tc::smem_desc(reinterpret_cast<char *>(Blo) + off, LBO, SBO);
            tc::mma_tf32(sm.tmem, ah, bh, IDESC, (chunk > 0 || st > 0) ? 1u : 0u);
            tc::mma_tf32(sm.tmem, ah, bl, IDESC, 1u);
            tc::mma_tf32(sm.tmem, al, bh, IDESC, 1u);
          }
          tc::mma_commit(sm.bar);
        }
      }
      ok = wait_mma<float, W>(sm) && ok;
      tc::fence_after_sync();
      const int sp = warp & 3, cq = warp >> 2;
      const int x = i0 + 32 * sp + lane;
#pragma unroll 1
      for (int c16 = 0; c16 < 4; ++c16) {
        float d[16];
        tc::tmem_ld16(sm.tmem + (uint32_t(32 * sp) << 16) + uint32_t(64 * cq + 16 * c16), d);
        if (x < M) {
#pragma unroll
          for (int q = 0; q < 8; ++q) {
            const int y = y0 + 32 * cq + 8 * c16 + q;
            if (y < N) E(x, y, mkc<float>(d[2 * q], d[2 * q + 1]));
          }
        }
      }
      tc::fence_before_sync();
      __syncthreads();
    }
  }
  return ok;
}

// gemm_nt on the tensor cores when the executor has them (float) and the
// product is large enough to fill the tiles, else on the SIMT path.
template <typename T, int NT, int W, class FP, class FQ, class FE>
__device__ bool gemm_nt_auto(int M, int N, int K, FP P, FQ Q, FE E, Smem<T, W> &sm) {
  if constexpr (sizeof(T) == 4) {
    if (sm.tc && M >= 64 && N >= 32 && K >= 16) return gemm_nt_tc<NT, W>(M, N, K, P, Q, E, sm);
  }
  gemm_nt<T, NT, W>(M, N, K, P, Q, E, sm);
  return true;
}

template <typename T, int NT, int W>
__device__ void finalize_bond(const TrajDev &tr, int k, cpx<T> *__restrict__ gk, cpx<T> *__restrict__ gk1,
                              const double *__restrict__ lamL, double *__restrict__ lamM,
                              const double *__restrict__ lamR, int cL, int cR, bool colmode, int ell, int c,
                              Work<T> &wk, Smem<T, W> &sm) {
  const int P = [&] {
    int p = 1;
    while (p < c) p <<= 1;
    return p;
  }();
  double *key = reinterpret_cast<double *>(sm.r0);
  int *pidx = reinterpret_cast<int *>(key + P);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  // vector norms (float64 accumulation)
  for (int j = warp; j < P; j += NT / 32) {
    T part = T(0);  // per-lane partial in the working precision, lanes summed in float64
    if (j < c) {
      const cpx<T> *a = wk.A + size_t(j) * ell;
      for (int i = lane; i < ell; i += 32) part += cabs2(a[i]);
    }
    double acc = double(part);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) {
      key[j] = (j < c) ? sqrt(acc) : -1.0;
      pidx[j] = j;
    }
  }
  __syncthreads();
  bitonic_desc<T, NT, W>(key, pidx, P);
  // norm of all singular values, normalise
  double part = 0.0;
  for (int j = threadIdx.x; j < c; j += NT) part += key[j] * key[j];
  const double norm1 = sqrt(block_sum<NT>(part, sm.red));
  // rank rule on s/||s||
  int mode = tr.trunc_mode;
  double eps = (mode == 2 || mode == 3) ? fabs(tr.cutoff) : 2.220446049250313e-16;
  // Exact zeros of the spectrum come out of the Jacobi sweeps at about
  // sqrt(ell)*eps_T relative to s_max (rounding of theta and of the
  // rotations).  Values below that floor are noise in any SVD (LAPACK's
  // included) and dividing by them (Gamma = U / Lambda) amplifies rounding,
  // so they are never kept.  The floor only matters for None/Const (the
  // reference's threshold is f64::EPSILON there); cutoffs >= 1e-12 are above it.
  eps = fmax(eps, rank_floor<T>(ell));
  int firstbad = c;
  for (int j = threadIdx.x; j < c; j += NT) {
    double s = key[j] / norm1;
    if (!is_normal_pos(s, eps)) firstbad = min(firstbad, j);
  }
  int nlead = block_min_int<NT>(firstbad, sm.ired);
  int rank;
  if (mode == 1) {
    rank = min(max(tr.chi_max, 1), nlead);
    if (rank < 1) rank = 1;  // all-zero spectrum: keep one vector instead of none
  } else if (mode == 3) {
    rank = max(1, min(tr.chi_max, nlead));
  } else {
    rank = max(nlead, 1);
  }
  if (rank > tr.cap) {
    if (threadIdx.x == 0) atomicOr(tr.status, ST_CAPACITY);
    rank = tr.cap;
  }
  double part2 = 0.0;
  for (int j = threadIdx.x; j < rank; j += NT) {
    double s = key[j] / norm1;
    part2 += s * s;
  }
  const double norm2 = sqrt(block_sum<NT>(part2, sm.red));
  // Per-value factors in the working precision (float64 only for these few
  // scalars): kept Schmidt values s2 (float64, stored as Lambda_k), 1/sigma,
  // 1/sigma^2 and s2^2 as T.
  for (int j = threadIdx.x; j < rank; j += NT) {
    double s1 = key[j] / norm1;
    double s2 = s1 / norm2;
    wk.s2[j] = s2;
    wk.perm[j] = pidx[j];
    wk.isig[j] = T(1.0 / key[j]);
    wk.isig2[j] = T(1.0 / (key[j] * key[j]));
    wk.w2[j] = T(s2 * s2);
  }
  // scl[0..cL): 1/Lambda_{k-1}[v]; scl[cap..cap+cR): norm2/Lambda_{k+1}[w]
  T *sclL = wk.scl, *sclR = wk.scl + tr.cap;
  for (int v = threadIdx.x; v < cL; v += NT) sclL[v] = T(1.0 / lamL[v]);
  for (int w = threadIdx.x; w < cR; w += NT) sclR[w] = T(norm2 / lamR[w]);
  __syncthreads();
  const int m = 2 * cL, nc = 2 * cR;
  const cpx<T> *A = wk.A, *T0 = wk.T0;
  const T *isig = wk.isig, *isig2 = wk.isig2, *w2 = wk.w2;
  const T *lLf = wk.lam3, *lRf = wk.lam3 + 2 * tr.cap;
  const int *perm = wk.perm;
  if (colmode) {
    // vectors = columns: U[:, j] = a_src / sigma (direct)
    for (size_t idx = threadIdx.x; idx < size_t(m) * rank; idx += NT) {
      int i = int(idx / rank), j = int(idx % rank);
      gk[idx] = cscale(A[size_t(perm[j]) * ell + i], isig[j] * sclL[i >> 1]);
    }
    // Vh[j][col] = sum_i conj(a_src[i]) theta[i][col] / sigma^2 (recovered)
    gemm_nt_auto<T, NT, W>(
        rank, nc, m,
        [&](int j, int i) {
          cpx<T> a = A[size_t(perm[j]) * ell + i];
          return mkc<T>(a.x, -a.y);
        },
        [&](int col, int i) { return T0[size_t(col) * m + i]; },
        [&](int j, int col, cpx<T> v) { gk1[size_t(j) * nc + col] = cscale(v, isig2[j] * sclR[col % cR]); }, sm);
  } else {
    // vectors = rows: Vh[j, :] = w_src / sigma (direct)
    for (size_t idx = threadIdx.x; idx < size_t(rank) * nc; idx += NT) {
      int j = int(idx / nc), col = int(idx % nc);
      gk1[idx] = cscale(A[size_t(perm[j]) * ell + col], isig[j] * sclR[col % cR]);
    }
    // U[i][j] = sum_col theta[i][col] conj(w_src[col]) / sigma^2 (recovered)
    gemm_nt_auto<T, NT, W>(
        m, rank, nc, [&](int i, int col) { return T0[size_t(i) * nc + col]; },
        [&](int j, int col) {
          cpx<T> a = A[size_t(perm[j]) * ell + col];
          return mkc<T>(a.x, -a.y);
        },
        [&](int i, int j, cpx<T> v) { gk[size_t(i) * rank + j] = cscale(v, isig2[j] * sclL[i >> 1]); }, sm);
  }
  __syncthreads();
  // local_renormalize(k) and (k+1) with the new Lambda_k = s2: per-thread
  // partial sums in the working precision, the block reduction in float64
  T pk = T(0), pk1 = T(0);
  for (size_t idx = threadIdx.x; idx < size_t(m) * rank; idx += NT) {
    int i = int(idx / rank), j = int(idx % rank);
    T l = lLf[i >> 1];
    pk += cabs2(gk[idx]) * (l * l) * w2[j];
  }
  for (size_t idx = threadIdx.x; idx < size_t(rank) * nc; idx += NT) {
    int j = int(idx / nc), w = int(idx % nc) % cR;
    T l = lRf[w];
    pk1 += cabs2(gk1[idx]) * w2[j] * (l * l);
  }
  double nk = double(pk), nk1 = double(pk1);
  block_sum2<NT>(nk, nk1, sm.red);
  const T ik = T(1.0 / sqrt(nk)), ik1 = T(1.0 / sqrt(nk1));
  for (size_t idx = threadIdx.x; idx < size_t(m) * rank; idx += NT) gk[idx] = cscale(gk[idx], ik);
  for (size_t idx = threadIdx.x; idx < size_t(rank) * nc; idx += NT) gk1[idx] = cscale(gk1[idx], ik1);
  for (int j = threadIdx.x; j < rank; j += NT) lamM[j] = wk.s2[j];
  if (threadIdx.x == 0) tr.chi[k + 1] = rank;
  __syncthreads();
}

// ---------------------------------------------------------- accessors
template <typename T>
__device__ __forceinline__ cpx<T> *gamma_slot(const TrajDev &tr, int k) {
  return reinterpret_cast<cpx<T> *>(tr.gamma) + size_t(k) * 2 * tr.cap * tr.cap;
}
__device__ __forceinline__ double *lam_slot(const TrajDev &tr, int s) { return tr.lam + size_t(s) * tr.cap; }

// In-place Cholesky S = L L^H of the n x n Hermitian matrix S (row-major,
// global scratch; the lower triangle becomes L).  Fails (returns false) when
// a pivot falls below `rel` times the original diagonal entry, i.e. when the
// rows behind S are far from orthonormal.
template <typename T, int NT, int W>
__device__ bool cholesky_lower(cpx<T> *__restrict__ S, int n, double rel, double *__restrict__ diag0,
                               Smem<T, W> &sm) {
  for (int i = threadIdx.x; i < n; i += NT) diag0[i] = double(S[size_t(i) * n + i].x);
  __syncthreads();
  for (int k = 0; k < n; ++k) {
    const double d = double(S[size_t(k) * n + k].x);
    if (!(d > rel * diag0[k]) || !(d > 0.0)) return false;  // uniform: every thread read the same value
    const T l = T(sqrt(d)), il = T(1.0 / sqrt(d));
    __syncthreads();
    for (int i = k + 1 + threadIdx.x; i < n; i += NT) S[size_t(i) * n + k] = cscale(S[size_t(i) * n + k], il);
    if (threadIdx.x == 0) S[size_t(k) * n + k] = mkc<T>(l, T(0));
    __syncthreads();
    const int rem = n - k - 1;
    for (int idx = threadIdx.x; idx < rem * rem; idx += NT) {
      const int i = k + 1 + idx / rem, j = k + 1 + idx % rem;
      if (j > i) continue;
      const cpx<T> li = S[size_t(i) * n + k], lj = S[size_t(j) * n + k];
      // S[i][j] -= L[i][k] conj(L[j][k])
      cpx<T> v = S[size_t(i) * n + j];
      v.x -= li.x * lj.x + li.y * lj.y;
      v.y -= li.y * lj.x - li.x * lj.y;
      S[size_t(i) * n + j] = v;
    }
    __syncthreads();
  }
  return true;
}

// Refactor through the LQ factor of the right block (local_refactor,
// mps.rs:846-880).  theta = X diag(Lambda_k) B with X = Lambda_{k-1} Gamma_k
// (m x chiM) and B = Gamma_{k+1} Lambda_{k+1} (chiM x nc).  With
// B B^H = L L^H, Q = L^{-1} B has orthonormal rows and theta = M Q,
// M = X diag(Lambda_k) L: the singular values and left vectors of theta are
// those of M (chiM columns), and Vh = U^H theta / sigma is recovered from
// theta itself.  In (near-)canonical form L is close to the identity, M has
// nearly orthogonal columns and the Jacobi sweeps converge in two or three
// passes.  Returns false (and leaves theta in wk.T0 untouched) when B is too
// far from orthonormal rows for the factorisation to be accurate.
template <typename T, int NT, int W>
__device__ bool refactor_lq(const cpx<T> *__restrict__ gk, const cpx<T> *__restrict__ gk1,
                            const T *__restrict__ lamL, const T *__restrict__ lamM,
                            const T *__restrict__ lamR, int cL, int cM, int cR, int cap, Work<T> &wk,
                            Smem<T, W> &sm) {
  const int m = 2 * cL, nc = 2 * cR;
  cpx<T> *S = wk.A + size_t(2) * cap * cap;  // chiM x chiM, after M's m x chiM region
  // S = B B^H
  gemm_nt_auto<T, NT, W>(
      cM, cM, nc, [&](int x, int col) { return cscale(gk1[size_t(x) * nc + col], lamR[col % cR]); },
      [&](int y, int col) {
        cpx<T> b = cscale(gk1[size_t(y) * nc + col], lamR[col % cR]);
        return mkc<T>(b.x, -b.y);
      },
      [&](int x, int y, cpx<T> v) { S[size_t(x) * cM + y] = v; }, sm);
  const double rel = sizeof(T) == 4 ? 0.1 : 1e-3;
  if (!cholesky_lower<T, NT, W>(S, cM, rel, wk.sig, sm)) return false;
  // M = X diag(Lambda_k) L, stored vector-contiguous: A[j*m + i] = M[i][j]
  cpx<T> *A = wk.A;
  gemm_nt_auto<T, NT, W>(
      m, cM, cM,
      [&](int i, int u) { return cscale(gk[size_t(i) * cM + u], lamL[i >> 1] * lamM[u]); },
      [&](int j, int u) { return u >= j ? S[size_t(u) * cM + j] : czero<T>(); },
      [&](int i, int j, cpx<T> v) { A[size_t(j) * m + i] = v; }, sm);
  return true;
}

// One bond operation on (k, k+1): gate != nullptr -> apply_unitary2, else local_refactor.
template <typename T, int NT, int W>
__device__ void bond_op(const TrajDev &tr, int k, const double *gate, Work<T> &wk, int max_sweeps, int scheme,
                        Smem<T, W> &sm) {
  const int cL = tr.chi[k], cM = tr.chi[k + 1], cR = tr.chi[k + 2];
  const int m = 2 * cL, nc = 2 * cR;
  cpx<T> *gk = gamma_slot<T>(tr, k), *gk1 = gamma_slot<T>(tr, k + 1);
  const double *lamL = lam_slot(tr, k), *lamR = lam_slot(tr, k + 2);
  double *lamM = lam_slot(tr, k + 1);
  long long c0 = clock64();
  // Lambda_{k-1}, Lambda_k, Lambda_{k+1} in the working precision (the state
  // keeps them in float64; the contraction multiplies in T)
  T *lLt = wk.lam3, *lMt = wk.lam3 + tr.cap, *lRt = wk.lam3 + 2 * tr.cap;
  for (int v = threadIdx.x; v < cL; v += NT) lLt[v] = T(lamL[v]);
  for (int u = threadIdx.x; u < cM; u += NT) lMt[u] = T(lamM[u]);
  for (int w = threadIdx.x; w < cR; w += NT) lRt[w] = T(lamR[w]);
  __syncthreads();
  // Refactors of a bond whose theta has more columns than its rank bound
  // chiM go through the LQ-reduced matrix M (m x chiM); gates and small
  // bonds take the direct path on theta.
  bool lq = false;
  // theta on the tensor cores when the CTA has them and the tiles are not
  // mostly padding; otherwise the SIMT contraction
  auto theta = [&](const double *g, cpx<T> *dst, cpx<T> *copy, bool cm) {
    if constexpr (sizeof(T) == 4) {
      if (sm.tc && m >= 64 && cR >= 16 && cM >= 8) {
        build_theta_tc<NT, W>(gk, gk1, lLt, lMt, lRt, cL, cM, cR, g, dst, copy, cm, sm);
        return;
      }
    }
    build_theta<T, NT, W>(gk, gk1, lLt, lMt, lRt, cL, cM, cR, g, dst, copy, cm, sm);
  };
  if (!gate && cM < nc && cM <= m) {
    theta(nullptr, wk.T0, wk.T0, true);
    lq = refactor_lq<T, NT, W>(gk, gk1, lLt, lMt, lRt, cL, cM, cR, tr.cap, wk, sm);
  }
  bool colmode;
  int ell, c;
  if (lq) {
    colmode = true;
    ell = m;
    c = cM;
  } else {
    colmode = m > nc;  // square: vectors = rows (coalesced theta stores)
    ell = colmode ? m : nc;
    c = colmode ? nc : m;
    theta(gate, wk.A, wk.T0, colmode);
  }
  long long c1 = clock64();
  long long cyc[4] = {0, 0, 0, 0};
  int sw = jacobi_svd<T, NT, W>(wk.A, ell, c, max_sweeps, sm, cyc, wk.sig, wk.perm, scheme);
  long long c2 = clock64();
  if (threadIdx.x == 0) {
    if (sw < 0) {
      atomicOr(tr.status, ST_NOT_CONVERGED);
      if (tr.stats) {
        atomicAdd(tr.stats + STAT_NONCONV, 1.0);
        atomicAdd(tr.stats + (lq ? STAT_NONCONV_LQ : STAT_NONCONV_DIRECT), double(c));
      }
    }
    if (tr.stats) {
      if (lq) atomicAdd(tr.stats + STAT_LQ_OPS, 1.0);
      const double a = double(m > nc ? m : nc), b = double(m > nc ? nc : m);
      double ft = 8.0 * m * double(cM) * nc + (gate ? 128.0 * cL * cR : 0.0);
      atomicAdd(tr.stats + STAT_FLOP_THETA, ft);
      atomicAdd(tr.stats + STAT_FLOP_SVD, 4.0 * (4.0 * a * a * b + 8.0 * a * b * b + 9.0 * b * b * b));
      atomicAdd(tr.stats + STAT_BOND_OPS, 1.0);
      atomicAdd(tr.stats + STAT_SWEEPS, double(sw < 0 ? max_sweeps : sw));
      // read the Gamma pair + Lambdas, write the new Gamma pair
      const double eb = double(sizeof(cpx<T>));
      atomicAdd(tr.stats + STAT_BYTES, eb * (2.0 * cL * cM + 2.0 * cM * cR) * 2.0 + 8.0 * (cL + cM + cR));
    }
  }
  finalize_bond<T, NT, W>(tr, k, gk, gk1, lamL, lamM, lamR, cL, cR, colmode, ell, c, wk, sm);
  if (sm.tc_fail) {  // a tensor-core wait gave up: the op's result is not trustworthy
    if (threadIdx.x == 0) atomicOr(tr.status, ST_BAD_INSTR);
    sm.tc_fail = false;
  }
  if (threadIdx.x == 0 && tr.stats) {
    atomicAdd(tr.stats + STAT_CYC_THETA, double(c1 - c0));
    atomicAdd(tr.stats + STAT_CYC_GRAM, double(cyc[0]));
    atomicAdd(tr.stats + STAT_CYC_ROT, double(cyc[1]));
    atomicAdd(tr.stats + STAT_CYC_UPDATE, double(cyc[2]));
    atomicAdd(tr.stats + STAT_CYC_FINAL, double(clock64() - c2));
    atomicAdd(tr.stats + STAT_BLOCK_STEPS, double(cyc[3]));
  }
}

// local_probs (mps.rs:1079-1134): p_s = sum L_{k-1}[v]^2 |G[v,s,u]|^2 L_k[u]^2
template <typename T, int NT, int W>
__device__ void site_probs(const TrajDev &tr, int k, double &p0, double &p1, Smem<T, W> &sm) {
  const int cL = tr.chi[k], cR = tr.chi[k + 1];
  const cpx<T> *g = gamma_slot<T>(tr, k);
  const double *lamL = lam_slot(tr, k), *lamR = lam_slot(tr, k + 1);
  // squared Lambdas in the working precision (shared scratch), per-thread
  // partial sums in T, block reduction in float64
  T *wl2 = reinterpret_cast<T *>(sm.r0), *wr2 = wl2 + cL;
  __syncthreads();
  for (int v = threadIdx.x; v < cL; v += NT) wl2[v] = T(lamL[v] * lamL[v]);
  for (int u = threadIdx.x; u < cR; u += NT) wr2[u] = T(lamR[u] * lamR[u]);
  __syncthreads();
  T b0 = T(0), b1 = T(0);
  const int tot = cL * 2 * cR;
  for (int idx = threadIdx.x; idx < tot; idx += NT) {
    int u = idx % cR, s = (idx / cR) & 1, v = idx / (2 * cR);
    T w = cabs2(g[idx]) * wl2[v] * wr2[u];
    if (s) b1 += w; else b0 += w;
  }
  double a0 = double(b0), a1 = double(b1);
  block_sum2<NT>(a0, a1, sm.red);
  p0 = a0;
  p1 = a1;
}

// sample_state + project (mps.rs:1427-1465)
template <typename T, int NT, int W>
__device__ void measure_site(const TrajDev &tr, int k, double u, int post, int *out_outcome, double *out_prob,
                             Smem<T, W> &sm) {
  double p0, p1;
  site_probs<T, NT, W>(tr, k, p0, p1, sm);
  int outcome;
  if (post >= 0)
    outcome = post;
  else
    outcome = (u < p0) ? 0 : 1;
  const double prob = outcome ? p1 : p0;
  const double sum = p0 + p1;
  if (threadIdx.x == 0) {
    if (tr.stats) {
      atomicAdd(tr.stats + STAT_MEAS, 1.0);
      atomicAdd(tr.stats + STAT_BYTES, double(sizeof(cpx<T>)) * 2.0 * 2.0 * tr.chi[k] * tr.chi[k + 1]);
    }
    if (out_outcome) *out_outcome = outcome;
    if (out_prob) *out_prob = prob;
    const double ptol = (sizeof(T) == 8) ? 1e-9 : 1e-4;
    if (!(fabs(sum - 1.0) <= ptol)) atomicOr(tr.status, ST_PROB_SUM);
  }
  const int cL = tr.chi[k], cR = tr.chi[k + 1];
  cpx<T> *g = gamma_slot<T>(tr, k);
  const T inv = T(1.0 / sqrt(prob));
  const int tot = cL * 2 * cR;
  for (int idx = threadIdx.x; idx < tot; idx += NT) {
    int s = (idx / cR) & 1;
    g[idx] = (s == outcome) ? cscale(g[idx], inv) : czero<T>();
  }
  __syncthreads();
}

// apply_unitary1 (mps.rs:1298-1314): Gamma_k[v,:,u] <- op Gamma_k[v,:,u]
template <typename T, int NT, int W>
__device__ void unitary1(const TrajDev &tr, int k, const double *op) {
  const int cL = tr.chi[k], cR = tr.chi[k + 1];
  cpx<T> *g = gamma_slot<T>(tr, k);
  cpx<T> o00 = mkc<T>(T(op[0]), T(op[1])), o01 = mkc<T>(T(op[2]), T(op[3]));
  cpx<T> o10 = mkc<T>(T(op[4]), T(op[5])), o11 = mkc<T>(T(op[6]), T(op[7]));
  for (int idx = threadIdx.x; idx < cL * cR; idx += NT) {
    int v = idx / cR, u = idx % cR;
    cpx<T> a = g[(v * 2 + 0) * cR + u], b = g[(v * 2 + 1) * cR + u];
    g[(v * 2 + 0) * cR + u] = cfma(o01, b, cmul(o00, a));
    g[(v * 2 + 1) * cR + u] = cfma(o11, b, cmul(o10, a));
  }
  __syncthreads();
}

// entropy_vn (mps.rs:1251-1261) / entropy_ry_schmidt (1268-1282), float64
template <int NT>
__device__ double bond_entropy(const TrajDev &tr, int b, double alpha, double *red) {
  const int cb = tr.chi[b + 1];
  const double *s = tr.lam + size_t(b + 1) * tr.cap;
  double acc = 0.0;
  for (int j = threadIdx.x; j < cb; j += NT) {
    double s2 = s[j] * s[j];
    if (alpha == 1.0)
      acc += -s2 * log(s2);
    else
      acc += pow(s2, alpha);
  }
  double tot = block_sum<NT>(acc, red);
  if (alpha == 1.0) return tot;
  return log(tot) / (1.0 - alpha);
}

template <typename T, int NT, int W>
__device__ void run_program(const LaunchArgs &la, const Instr *prog, const Item &it, Work<T> &wk, Smem<T, W> &sm) {
  const TrajDev tr = la.trajs[it.traj];
  for (int pc = 0; pc < it.len; ++pc) {
    const Instr in = prog[it.off + pc];
    switch (in.op) {
      case OP_GATE:
        bond_op<T, NT, W>(tr, in.k, la.gates + size_t(in.a) * 32, wk, la.max_sweeps, la.jacobi_scheme, sm);
        break;
      case OP_REFACTOR:
        bond_op<T, NT, W>(tr, in.k, nullptr, wk, la.max_sweeps, la.jacobi_scheme, sm);
        break;
      case OP_MEAS:
        measure_site<T, NT, W>(tr, in.k, la.us[in.a], in.b, la.outcomes + in.a, la.probs + in.a, sm);
        break;
      case OP_ENTROPY: {
        double e = bond_entropy<NT>(tr, in.k, 1.0, sm.red);
        if (threadIdx.x == 0) la.ents[in.a] = e;
        __syncthreads();
        break;
      }
      case OP_RENYI: {
        double e = bond_entropy<NT>(tr, in.k, la.us[in.b], sm.red);
        if (threadIdx.x == 0) la.ents[in.a] = e;
        __syncthreads();
        break;
      }
      case OP_UNI1:
        unitary1<T, NT, W>(tr, in.k, la.gates + size_t(in.a) * 32);
        break;
      case OP_PROBS: {
        double p0, p1;
        site_probs<T, NT, W>(tr, in.k, p0, p1, sm);
        if (threadIdx.x == 0) {
          la.pout[2 * in.a] = p0;
          la.pout[2 * in.a + 1] = p1;
        }
        __syncthreads();
        break;
      }
      case OP_NOP:
        break;
      default:
        if (threadIdx.x == 0) atomicOr(tr.status, ST_BAD_INSTR);
        break;
    }
  }
}

}  // namespace tn
