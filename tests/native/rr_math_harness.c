/* Test harness for csrc/common/rr_math.h on the host: the CPU tests compile
 * it with gcc -ffp-contract=off (C99, as the oracle is built) and call it
 * through ctypes. */
#include <stdint.h>

#include "../../rils-rols_gb300/csrc/common/rr_math.h"

/* op: 0 exp, 1 log, 2 sin, 3 cos, 4 pow (b used) */
void rr_apply(int op, const double* a, const double* b, int64_t n, double* out) {
  for (int64_t i = 0; i < n; ++i) {
    switch (op) {
      case 0: out[i] = rr_exp(a[i]); break;
      case 1: out[i] = rr_log(a[i]); break;
      case 2: out[i] = rr_sin(a[i]); break;
      case 3: out[i] = rr_cos(a[i]); break;
      default: out[i] = rr_pow(a[i], b[i]); break;
    }
  }
}
