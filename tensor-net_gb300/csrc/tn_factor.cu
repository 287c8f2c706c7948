// tn_factor.cu -- MPS::from_vector / factorize (mps.rs:448-550) on the GPU.
//
// The dense state (2^n complex128, s_0 most significant) is normalised, then
// factorised site by site, left to right: the remainder Q (chi_{k-1} rows of
// 2^(n-k) amplitudes) is read as the m x N matrix M with m = 2 chi_{k-1} and
// N = 2^(n-k-1) (a free reshape of the row-major buffer), M = U S V^H, and
//   Gamma_k = U[:, :rank] as (chi_{k-1}, 2, rank), divided by Lambda_{k-1} on
//             its first axis (not at k = 0),
//   Lambda_k = the kept Schmidt values of process_svd (mps.rs:236-293),
//   Q <- rows j < rank of S V^H / ||S||  (process_svd's q_j = V^H_j s_j/||s||).
// The last Gamma is Q as (chi_{n-2}, 2, 1) divided by Lambda_{n-2}.
//
// The SVD is a one-sided Jacobi over the ROWS of M in float64 (Hestenes'
// method, the published algorithm: plane rotations that orthogonalise pairs
// of vectors until every pair is orthogonal to a relative tolerance).  After
// convergence the rows of R M are orthogonal, R the product of the
// rotations: their norms are the singular values, the rows themselves
// S V^H, and U = R^H.  One launch per round of disjoint pairs (the
// round-robin "circle" ordering, m - 1 rounds per sweep), one warp per pair;
// the host reads a rotated-anything flag after each sweep.  Rows whose
// squared norm is below 1e-30 are numerical zeros (the remainder's squared
// norm lies between 1/m and 1) and are left out of the rotations; they end
// below the EPS cutoff of the rank rule.
//
// This is an initialisation path (validation exports and prepared initial
// states), sized for n <= 20 (m <= 2048 rows, 2^20 amplitudes); the work per
// site is O(m^2 N) per sweep, which stays below a second per site there.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "tn_internal.h"
#include "tn_mps.h"

namespace {

constexpr int kFvMaxQubits = 20;
constexpr int kFvMaxRows = 2048;    // 2 * 2^(20/2)
constexpr int kFvRoundThreads = 256;
constexpr int kFvMaxSweeps = 60;
constexpr double kFvZeroRel = 1e-30;

__device__ __forceinline__ double warp_sum_bcast(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return __shfl_sync(0xffffffffu, v, 0);
}

// ||psi|| in a fixed order (one CTA of 1024 threads), then psi /= ||psi||.
__global__ void k_fv_norm(double2 *psi, uint64_t len, double *norm_out) {
  __shared__ double red[1024];
  double acc = 0.0;
  for (uint64_t i = threadIdx.x; i < len; i += blockDim.x) {
    const double2 z = psi[i];
    acc += z.x * z.x + z.y * z.y;
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  const double nrm = sqrt(red[0]);
  if (threadIdx.x == 0) *norm_out = nrm;
  if (!(nrm > 0.0) || !isfinite(nrm)) return;
  for (uint64_t i = threadIdx.x; i < len; i += blockDim.x) {
    double2 z = psi[i];
    z.x /= nrm;
    z.y /= nrm;
    psi[i] = z;
  }
}

__global__ void k_fv_eye(double2 *r, int m) {
  const uint64_t total = uint64_t(m) * m;
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < total;
       i += uint64_t(gridDim.x) * blockDim.x) {
    const bool diag = (i / m) == (i % m);
    r[i] = make_double2(diag ? 1.0 : 0.0, 0.0);
  }
}

// One round of the circle ordering over mp (even) players: pair 0 is
// (round, mp - 1), pair w > 0 is ((round + w) mod (mp - 1), (round - w) mod (mp - 1)).
// Each warp orthogonalises its pair of rows of q (length nq) and applies the
// same rotation to the rows of r (length m).
__global__ void k_fv_round(double2 *q, double2 *r, int m, int mp, uint64_t nq, int round, double tol,
                           double zero2, int *rotated) {
  const int warp = int((blockIdx.x * uint64_t(blockDim.x) + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (warp >= mp / 2) return;
  const int ring = mp - 1;
  int a, b;
  if (warp == 0) {
    a = round;
    b = mp - 1;
  } else {
    a = (round + warp) % ring;
    b = (round - warp + ring) % ring;
  }
  if (a >= m || b >= m) return;
  const int p = a < b ? a : b, s = a < b ? b : a;
  double2 *rp = q + uint64_t(p) * nq, *rs = q + uint64_t(s) * nq;
  double al = 0.0, be = 0.0, gr = 0.0, gi = 0.0;
  for (uint64_t i = lane; i < nq; i += 32) {
    const double2 x = rp[i], y = rs[i];
    al += x.x * x.x + x.y * x.y;
    be += y.x * y.x + y.y * y.y;
    gr += x.x * y.x + x.y * y.y;  // conj(x) * y
    gi += x.x * y.y - x.y * y.x;
  }
  al = warp_sum_bcast(al);
  be = warp_sum_bcast(be);
  gr = warp_sum_bcast(gr);
  gi = warp_sum_bcast(gi);
  if (al < zero2 || be < zero2) return;
  const double g = hypot(gr, gi);
  if (!(g > tol * sqrt(al) * sqrt(be))) return;
  // Rotation of the 2x2 Gram [[al, g], [g, be]] after phasing row s by
  // w = conj(gamma)/|gamma|: t = sign(zeta)/(|zeta| + sqrt(1 + zeta^2)).
  const double zeta = (be - al) / (2.0 * g);
  const double t = (zeta >= 0.0 ? 1.0 : -1.0) / (fabs(zeta) + hypot(1.0, zeta));
  const double c = 1.0 / sqrt(1.0 + t * t), sn = c * t;
  const double wr = gr / g, wi = -gi / g;
  for (uint64_t i = lane; i < nq; i += 32) {
    const double2 x = rp[i], y = rs[i];
    const double yr = wr * y.x - wi * y.y, yi = wr * y.y + wi * y.x;
    rp[i] = make_double2(c * x.x - sn * yr, c * x.y - sn * yi);
    rs[i] = make_double2(sn * x.x + c * yr, sn * x.y + c * yi);
  }
  double2 *up = r + uint64_t(p) * m, *us = r + uint64_t(s) * m;
  for (int i = lane; i < m; i += 32) {
    const double2 x = up[i], y = us[i];
    const double yr = wr * y.x - wi * y.y, yi = wr * y.y + wi * y.x;
    up[i] = make_double2(c * x.x - sn * yr, c * x.y - sn * yi);
    us[i] = make_double2(sn * x.x + c * yr, sn * x.y + c * yi);
  }
  if (lane == 0) atomicOr(rotated, 1);
}

// Stores the complex value (re, im) as element i of a Gamma slot in the
// layout of precision prec (0: complex128, 1: complex64, 2: double-float).
__device__ void store_elem(void *gamma, int prec, size_t i, double re, double im) {
  if (prec == 0) {
    reinterpret_cast<double2 *>(gamma)[i] = make_double2(re, im);
  } else if (prec == 2) {
    const float rh = __double2float_rn(re), ih = __double2float_rn(im);
    reinterpret_cast<float4 *>(gamma)[i] =
        make_float4(rh, __double2float_rn(re - double(rh)), ih, __double2float_rn(im - double(ih)));
  } else {
    reinterpret_cast<float2 *>(gamma)[i] = make_float2(float(re), float(im));
  }
}

__device__ bool fv_normal(double x) { return isfinite(x) && x != 0.0 && fabs(x) >= 2.2250738585072014e-308; }

// Schmidt values, rank rule and the site's outputs (one CTA of 1024 threads).
__global__ void k_fv_finish(const double2 *q, const double2 *r, double2 *qn, int m, uint64_t nq, int k,
                            tn::TrajDev tr, int prec, int *rank_out) {
  __shared__ double sv[kFvMaxRows];
  __shared__ int perm[kFvMaxRows];
  __shared__ double s_snorm, s_norm2;
  __shared__ int s_rank;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
  for (int j = warp; j < m; j += nwarps) {
    const double2 *row = q + uint64_t(j) * nq;
    double acc = 0.0;
    for (uint64_t i = lane; i < nq; i += 32) acc += row[i].x * row[i].x + row[i].y * row[i].y;
    acc = warp_sum_bcast(acc);
    if (lane == 0) sv[j] = sqrt(acc);
  }
  __syncthreads();
  // descending order, ties by row index
  for (int j = threadIdx.x; j < m; j += blockDim.x) {
    int rk = 0;
    const double x = sv[j];
    for (int i = 0; i < m; ++i) rk += (sv[i] > x || (sv[i] == x && i < j)) ? 1 : 0;
    perm[rk] = j;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double tot = 0.0;
    for (int j = 0; j < m; ++j) tot += sv[perm[j]] * sv[perm[j]];
    const double snorm = sqrt(tot);
    // process_svd's rank rule on s / ||s|| (mps.rs:250-274)
    const bool has_cut = tr.trunc_mode == TN_TRUNC_CUTOFF || tr.trunc_mode == TN_TRUNC_BOTH;
    // values below the rounding noise of the rotated rows (about sqrt(len) eps
    // relative) are not kept, as in the bond operations: an exact low-rank
    // state would otherwise keep a noise value and divide Gamma by it
    const double noise = 4.0 * sqrt(double(uint64_t(m) > nq ? uint64_t(m) : nq)) * 2.220446049250313e-16;
    const double eps = fmax(has_cut ? fabs(tr.cutoff) : 2.220446049250313e-16, noise);
    // at most min(m, N) singular values, as a full SVD of the m x N matrix has
    const int lim = uint64_t(m) < nq ? m : int(nq);
    int lead = 0;
    while (lead < lim) {
      const double x = sv[perm[lead]] / snorm;
      if (!fv_normal(x) || !(x > eps)) break;
      ++lead;
    }
    int rank;
    if (tr.trunc_mode == TN_TRUNC_CONST) {
      rank = min(max(tr.chi_max, 1), lead);
    } else if (tr.trunc_mode == TN_TRUNC_BOTH) {
      rank = max(1, min(tr.chi_max, lead));
    } else {
      rank = max(lead, 1);
    }
    double n2 = 0.0;
    for (int j = 0; j < rank; ++j) {
      const double x = sv[perm[j]] / snorm;
      n2 += x * x;
    }
    s_snorm = snorm;
    s_norm2 = sqrt(n2);
    s_rank = (rank <= tr.cap && rank <= kFvMaxRows / 2) ? rank : -1;
  }
  __syncthreads();
  const int rank = s_rank;
  if (threadIdx.x == 0) *rank_out = rank;
  if (rank < 0) return;
  const double snorm = s_snorm, norm2 = s_norm2;
  double *lam = tr.lam + size_t(k + 1) * tr.cap;
  for (int j = threadIdx.x; j < rank; j += blockDim.x) lam[j] = (sv[perm[j]] / snorm) / norm2;
  if (threadIdx.x == 0) tr.chi[k + 1] = rank;
  // Gamma_k[v, s, j] = conj(R[perm[j], 2v + s]) / Lambda_{k-1}[v]
  const int udim = m / 2;
  const double *lam_prev = tr.lam + size_t(k) * tr.cap;
  const size_t slot = size_t(2) * tr.cap * tr.cap;
  const int cnt = udim * 2 * rank;
  for (int idx = threadIdx.x; idx < cnt; idx += blockDim.x) {
    const int j = idx % rank, row = idx / rank;  // row = 2v + s
    const double2 x = r[uint64_t(perm[j]) * m + row];
    double vr = x.x, vi = -x.y;
    if (k > 0) {
      const double l = lam_prev[row >> 1];
      vr /= l;
      vi /= l;
    }
    store_elem(tr.gamma, prec, size_t(k) * slot + idx, vr, vi);
  }
  // next remainder: rows j < rank of R M, divided by ||s||
  const uint64_t total = uint64_t(rank) * nq;
  for (uint64_t i = threadIdx.x; i < total; i += blockDim.x) {
    const uint64_t j = i / nq, c = i % nq;
    const double2 x = q[uint64_t(perm[j]) * nq + c];
    qn[i] = make_double2(x.x / snorm, x.y / snorm);
  }
}

// Last site: Gamma_{n-1}[v, s, 0] = Q[v, s] / Lambda_{n-2}[v]; the edge
// Lambdas and bond dimensions.  n == 1: Gamma_0 = psi.
__global__ void k_fv_last(const double2 *q, int udim, int n, tn::TrajDev tr, int prec) {
  const size_t slot = size_t(2) * tr.cap * tr.cap;
  const double *lam_prev = tr.lam + size_t(n - 1) * tr.cap;
  for (int idx = threadIdx.x; idx < 2 * udim; idx += blockDim.x) {
    double2 x = q[idx];
    if (n > 1) {
      const double l = lam_prev[idx >> 1];
      x.x /= l;
      x.y /= l;
    }
    store_elem(tr.gamma, prec, size_t(n - 1) * slot + idx, x.x, x.y);
  }
  if (threadIdx.x == 0) {
    tr.lam[0] = 1.0;
    tr.lam[size_t(n) * tr.cap] = 1.0;
    tr.chi[0] = 1;
    tr.chi[n] = 1;
    if (n == 1) tr.chi[1] = 1;
  }
}

struct Scratch {
  void *p = nullptr;
  ~Scratch() {
    if (p) cudaFree(p);
  }
};

#define FV_CK(call)                                        \
  do {                                                     \
    cudaError_t e__ = (call);                              \
    if (e__ != cudaSuccess) {                              \
      tn::set_last_error(#call, e__);                      \
      return e__ == cudaErrorMemoryAllocation ? TN_ERR_OOM : TN_ERR_CUDA; \
    }                                                      \
  } while (0)

int factorize(const tn::TrajDev &tr, int prec, const double *state, uint64_t len, cudaStream_t st) {
  const int n = tr.n;
  Scratch sa, sb, sr, sf;
  FV_CK(cudaMalloc(&sa.p, len * sizeof(double2)));
  FV_CK(cudaMalloc(&sb.p, len * sizeof(double2)));
  const int mmax = std::min(kFvMaxRows, 2 * tr.cap);
  FV_CK(cudaMalloc(&sr.p, size_t(mmax) * mmax * sizeof(double2)));
  FV_CK(cudaMalloc(&sf.p, 4 * sizeof(double)));
  double2 *qa = static_cast<double2 *>(sa.p), *qb = static_cast<double2 *>(sb.p);
  double2 *rm = static_cast<double2 *>(sr.p);
  double *dnorm = static_cast<double *>(sf.p);
  int *dflag = reinterpret_cast<int *>(dnorm + 1);
  int *drank = reinterpret_cast<int *>(dnorm + 2);
  FV_CK(cudaMemcpyAsync(qa, state, len * sizeof(double2), cudaMemcpyHostToDevice, st));
  k_fv_norm<<<1, 1024, 0, st>>>(qa, len, dnorm);
  FV_CK(cudaGetLastError());
  double norm = 0.0;
  FV_CK(cudaMemcpyAsync(&norm, dnorm, sizeof(double), cudaMemcpyDeviceToHost, st));
  FV_CK(cudaStreamSynchronize(st));
  if (!(norm > 0.0) || !std::isfinite(norm)) return TN_ERR_INVALID_ARG;
  int udim = 1;
  for (int k = 0; k + 1 < n; ++k) {
    const int m = 2 * udim;
    const uint64_t nq = len >> (k + 1);
    if (m > mmax) return TN_ERR_CAPACITY;
    const double tol = 1e-14 * std::max(1.0, std::sqrt(double(nq) / 1024.0));
    k_fv_eye<<<std::max(1, std::min(1024, (m * m + 255) / 256)), 256, 0, st>>>(rm, m);
    FV_CK(cudaGetLastError());
    const int mp = m + (m & 1);
    const int pairs = mp / 2;
    const int grid = (pairs * 32 + kFvRoundThreads - 1) / kFvRoundThreads;
    bool converged = false;
    for (int sweep = 0; sweep < kFvMaxSweeps && !converged; ++sweep) {
      FV_CK(cudaMemsetAsync(dflag, 0, sizeof(int), st));
      for (int round = 0; round < mp - 1; ++round)
        k_fv_round<<<grid, kFvRoundThreads, 0, st>>>(qa, rm, m, mp, nq, round, tol, kFvZeroRel, dflag);
      FV_CK(cudaGetLastError());
      int flag = 0;
      FV_CK(cudaMemcpyAsync(&flag, dflag, sizeof(int), cudaMemcpyDeviceToHost, st));
      FV_CK(cudaStreamSynchronize(st));
      converged = flag == 0;
    }
    if (!converged) return TN_ERR_NOT_CONVERGED;
    k_fv_finish<<<1, 1024, 0, st>>>(qa, rm, qb, m, nq, k, tr, prec, drank);
    FV_CK(cudaGetLastError());
    int rank = 0;
    FV_CK(cudaMemcpyAsync(&rank, drank, sizeof(int), cudaMemcpyDeviceToHost, st));
    FV_CK(cudaStreamSynchronize(st));
    if (rank < 1) return TN_ERR_CAPACITY;
    std::swap(qa, qb);
    udim = rank;
  }
  k_fv_last<<<1, 256, 0, st>>>(qa, udim, n, tr, prec);
  FV_CK(cudaGetLastError());
  FV_CK(cudaStreamSynchronize(st));
  return TN_OK;
}

}  // namespace

extern "C" {

int tn_mps_from_vector(uint32_t n, const double *state, uint64_t len, const tn_trunc *trunc, int32_t precision,
                       uint32_t chi_cap, tn_mps **out) {
  if (!out) return TN_ERR_INVALID_ARG;
  *out = nullptr;
  if (n == 0) return TN_ERR_EMPTY_SYSTEM;
  if (!state || n > uint32_t(kFvMaxQubits)) return TN_ERR_INVALID_ARG;
  if (len != (uint64_t(1) << n)) return TN_ERR_STATE_SHAPE;
  // bond capacity: chi_cap, else chi_max for CONST/BOTH, else every Schmidt rank of n qubits
  const uint32_t full = uint32_t(1) << (n / 2);
  uint32_t cap = full;
  if (chi_cap) {
    cap = std::min(chi_cap, full);
  } else if (trunc && (trunc->mode == TN_TRUNC_CONST || trunc->mode == TN_TRUNC_BOTH)) {
    cap = std::min(std::max<uint32_t>(1, trunc->chi_max), full);
  }
  tn_mps *m = nullptr;
  if (int s = tn_mps_new_qubits(n, trunc, precision, cap, &m)) return s;
  tn::MpsView v{};
  int s = tn::mps_view(m, &v);
  tn::TrajDev tr{};
  if (s == TN_OK) {
    cudaError_t e = cudaMemcpyAsync(&tr, v.dtraj, sizeof(tn::TrajDev), cudaMemcpyDeviceToHost, v.st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(v.st);
    if (e != cudaSuccess) {
      tn::set_last_error("read handle", e);
      s = TN_ERR_CUDA;
    }
  }
  if (s == TN_OK) s = factorize(tr, v.prec, state, len, v.st);
  if (s != TN_OK) {
    tn_mps_free(m);
    return s;
  }
  *out = m;
  return TN_OK;
}

}  // extern "C"
