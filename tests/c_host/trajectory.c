/* A plain C99 host of the C ABI (include/tn_mps.h): one seeded Haar
 * brickwork trajectory through tn_mps_apply_bilayer, printing the half-chain
 * entropy after every layer ("layer t entropy e" lines, %.17g).  Exit codes:
 * 0 done, 3 no CUDA device (the library refuses loudly), 1 any other error.
 * Usage: trajectory n depth p chi_max seed */
#include <stdio.h>
#include <stdlib.h>

#include "tn_mps.h"

int main(int argc, char **argv) {
  if (argc != 6) {
    fprintf(stderr, "usage: %s n depth p chi_max seed\n", argv[0]);
    return 1;
  }
  const uint32_t n = (uint32_t)strtoul(argv[1], NULL, 10), depth = (uint32_t)strtoul(argv[2], NULL, 10);
  const double p = strtod(argv[3], NULL);
  const uint32_t chi = (uint32_t)strtoul(argv[4], NULL, 10);
  const uint64_t seed = strtoull(argv[5], NULL, 10);
  if (n < 2 || n > 64) return 1;
  tn_trunc tr;
  tr.mode = TN_TRUNC_BOTH;
  tr.chi_max = chi;
  tr.cutoff = 1e-12;
  tn_mps *m = NULL;
  int s = tn_mps_new_qubits(n, &tr, TN_PREC_F64, 0, &m);
  if (s == TN_ERR_NO_DEVICE) {
    printf("%s\n", tn_status_string(s));
    return 3;
  }
  if (s != TN_OK) {
    fprintf(stderr, "tn_mps_new_qubits: %s (%s)\n", tn_status_string(s), tn_last_error());
    return 1;
  }
  uint32_t gk[64], mk[64], ng = 0, nm = 0, ok[64], nout = 0;
  double gates[32 * 33], us[64], probs[64], e = 0.0;
  int32_t oc[64];
  for (uint32_t t = 0; t < depth; ++t) {
    s = tn_gen_layer(seed, 0, t, n, p, gk, gates, &ng, mk, us, &nm);
    if (s == TN_OK) s = tn_mps_apply_bilayer(m, gk, gates, ng, mk, nm, us, ok, oc, probs, &nout);
    if (s == TN_OK) s = tn_mps_entropy_vn(m, n / 2 - 1, &e);
    if (s != TN_OK) {
      fprintf(stderr, "layer %u: %s (%s)\n", t, tn_status_string(s), tn_last_error());
      tn_mps_free(m);
      return 1;
    }
    printf("layer %u entropy %.17g measured %u\n", t, e, nout);
  }
  int32_t st = 0;
  tn_mps_device_status(m, &st);
  tn_mps_free(m);
  return st == 0 ? 0 : 1;
}
