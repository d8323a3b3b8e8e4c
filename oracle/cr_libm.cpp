// Test infrastructure only: the correctly rounded log/exp/pow (and atan/cos) of the CUDA path
// (epic_gb300/csrc/dd_math.cuh, host-compiled) behind C entry points for libepicport_cr.so.
#define __host__
#define __device__
#define __forceinline__ inline
#include "../epic_gb300/csrc/dd_math.cuh"

namespace {
const epic::MathTable &table() {
  static const epic::MathTable *t = [] {
    auto *p = new epic::MathTable;
    epic::fill_math_table(*p);
    return p;
  }();
  return *t;
}
}  // namespace

extern "C" double epic_cr_log(double x) { return epic::cr_log(x, table()); }
extern "C" double epic_cr_exp(double x) { return epic::cr_exp(x, table()); }
extern "C" double epic_cr_pow(double x, double y) { return epic::cr_pow(x, y, table()); }
extern "C" double epic_cr_atan(double x) { return epic::cr_atan(x, table()); }
extern "C" double epic_cr_cos(double x) { return epic::cr_cos(x, table()); }
