// tn_gen.cpp -- seeded synthetic inputs: Haar-random U(4) gates and
// measurement uniforms for brickwork layers.
//
// Counter-based: every number is a pure function of (seed, traj, layer, site,
// purpose, index), so a trajectory's inputs do not depend on which other
// trajectories are generated or in what order.  The mixer is SplitMix64
// (Steele, Lea, Flood 2014); normals come from the Box-Muller transform
// (Box & Muller 1958).  The Haar construction restates gate::haar
// (tensor-net/lib/gate.rs:888-909): a complex Ginibre matrix filled row-major
// with (re, im) standard normals, QR, and column j divided by r_jj/|r_jj|.
// The QR here is modified Gram-Schmidt with one re-orthogonalisation pass,
// which yields the same Q (the unique one with a positive real R diagonal).
#include <cmath>
#include <cstdint>
#include <cstring>

#include "tn_mps.h"

namespace {

inline uint64_t mix64(uint64_t z) {
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

enum Purpose : uint64_t { P_GATE = 1, P_LOC = 2, P_OUT = 3 };

inline uint64_t key(uint64_t seed, uint64_t traj, uint32_t layer, uint32_t site, uint64_t purpose, uint64_t idx) {
  uint64_t h = mix64(seed ^ 0x5851f42d4c957f2dull);
  h = mix64(h ^ traj);
  h = mix64(h ^ ((uint64_t(layer) << 32) | site));
  h = mix64(h ^ ((purpose << 56) | idx));
  return h;
}

// uniform in [0, 1) with 53 random bits
inline double unif(uint64_t k) { return double(k >> 11) * (1.0 / 9007199254740992.0); }

void normal_pair(uint64_t k, double &z0, double &z1) {
  const double u1 = 1.0 - unif(mix64(k ^ 0x1ull));  // (0, 1]
  const double u2 = unif(mix64(k ^ 0x2ull));
  const double r = std::sqrt(-2.0 * std::log(u1));
  const double th = 6.283185307179586 * u2;
  z0 = r * std::cos(th);
  z1 = r * std::sin(th);
}

struct C {
  double r, i;
};
inline C cmul(C a, C b) { return {a.r * b.r - a.i * b.i, a.r * b.i + a.i * b.r}; }
inline C cconj(C a) { return {a.r, -a.i}; }

}  // namespace

extern "C" {

int tn_haar_u4(const double *z, double *out) {
  if (!z || !out) return TN_ERR_INVALID_ARG;
  C a[4][4];  // a[row][col]
  for (int r = 0; r < 4; ++r)
    for (int c = 0; c < 4; ++c) a[r][c] = {z[2 * (r * 4 + c)], z[2 * (r * 4 + c) + 1]};
  C q[4][4];
  for (int j = 0; j < 4; ++j) {
    C v[4];
    for (int r = 0; r < 4; ++r) v[r] = a[r][j];
    for (int pass = 0; pass < 2; ++pass) {
      for (int i = 0; i < j; ++i) {
        C d{0.0, 0.0};  // q_i^H v
        for (int r = 0; r < 4; ++r) {
          C t = cmul(cconj(q[r][i]), v[r]);
          d.r += t.r;
          d.i += t.i;
        }
        for (int r = 0; r < 4; ++r) {
          C t = cmul(d, q[r][i]);
          v[r].r -= t.r;
          v[r].i -= t.i;
        }
      }
    }
    double nrm = 0.0;
    for (int r = 0; r < 4; ++r) nrm += v[r].r * v[r].r + v[r].i * v[r].i;
    nrm = std::sqrt(nrm);
    if (!(nrm > 0.0)) return TN_ERR_INVALID_ARG;
    for (int r = 0; r < 4; ++r) q[r][j] = {v[r].r / nrm, v[r].i / nrm};
  }
  for (int r = 0; r < 4; ++r)
    for (int c = 0; c < 4; ++c) {
      out[2 * (r * 4 + c)] = q[r][c].r;
      out[2 * (r * 4 + c) + 1] = q[r][c].i;
    }
  return TN_OK;
}

int tn_gen_layer(uint64_t seed, uint64_t traj, uint32_t layer, uint32_t n, double p, uint32_t *gate_ks,
                 double *gates, uint32_t *ng, uint32_t *meas_ks, double *us, uint32_t *nm) {
  if (n == 0) return TN_ERR_EMPTY_SYSTEM;
  uint32_t g = 0;
  // TileQ2::new(n, offs) (circuit.rs:527-531), offs = layer odd (workspace/lib/haar.rs:285)
  for (uint32_t k = (layer & 1u); k + 1 < n; k += 2) {
    if (gate_ks) gate_ks[g] = k;
    if (gates) {
      double z[32];
      for (int e = 0; e < 16; ++e) {
        double a, b;
        normal_pair(key(seed, traj, layer, k, P_GATE, uint64_t(e)), a, b);
        z[2 * e] = a;
        z[2 * e + 1] = b;
      }
      if (int s = tn_haar_u4(z, gates + size_t(g) * 32)) return s;
    }
    ++g;
  }
  if (ng) *ng = g;
  // uniform_meas (circuit.rs:580-584): qubit measured iff u_loc < p
  uint32_t m = 0;
  for (uint32_t k = 0; k < n; ++k) {
    const double uloc = unif(key(seed, traj, layer, k, P_LOC, 0));
    if (uloc < p) {
      if (meas_ks) meas_ks[m] = k;
      if (us) us[m] = unif(key(seed, traj, layer, k, P_OUT, 0));
      ++m;
    }
  }
  if (nm) *nm = m;
  return TN_OK;
}

// The Ginibre sample behind gate g of a layer, for checking tn_haar_u4
// against an independent QR.
int tn_gen_ginibre(uint64_t seed, uint64_t traj, uint32_t layer, uint32_t site, double *z) {
  if (!z) return TN_ERR_INVALID_ARG;
  for (int e = 0; e < 16; ++e) {
    double a, b;
    normal_pair(key(seed, traj, layer, site, P_GATE, uint64_t(e)), a, b);
    z[2 * e] = a;
    z[2 * e + 1] = b;
  }
  return TN_OK;
}

}  // extern "C"
