// Test harness for csrc/common/df32.h on the host: the CPU tests compile it
// with g++ -ffp-contract=off and call it through ctypes.
#include <cstdint>

#include "../../rils-rols_gb300/csrc/common/df32.h"

extern "C" {

// op: 0 add, 1 sub, 2 mul, 3 div, 4 sqrt, 5 exp, 6 log, 7 sin, 8 cos,
// 9 div by the reciprocal form (dfl_div_nc)
// a, b: n doubles each, converted to double-floats; out: n doubles (hi + lo)
void df32_apply(int op, const double* a, const double* b, int64_t n, double* out) {
  for (int64_t i = 0; i < n; ++i) {
    const dfl x = dfl_from_double(a[i]);
    const dfl y = dfl_from_double(b ? b[i] : 0.0);
    dfl r;
    switch (op) {
      case 0: r = dfl_add(x, y); break;
      case 1: r = dfl_sub(x, y); break;
      case 2: r = dfl_mul(x, y); break;
      case 3: r = dfl_div(x, y); break;
      case 4: r = dfl_sqrt(x); break;
      case 5: r = dfl_exp(x); break;
      case 6: r = dfl_log(x); break;
      case 7: r = dfl_sin(x); break;
      case 9: r = dfl_div_nc(x, y); break;
      default: r = dfl_cos(x); break;
    }
    out[i] = dfl_to_double(r);
  }
}

}
