// Host build of the weight primitives of ts_common.h, for the CPU tests.
#include "ts_common.h"

static const double kTab[64] = {TS_EXP2_TABLE_VALUES};
static const float kTabFF[128] = {TS_EXP2_FF_TABLE_VALUES};

extern "C" double host_exp(double x) { return ts::ts_exp64(x, kTab); }
extern "C" double host_div(double a, double b) { return ts::ts_div_markstein(a, b, 1.0 / b); }

// In-order sum of every value four times through ts_add4_rn.
extern "C" double host_sum4_int(const double *d, int n) {
  uint64_t acc = 0;
  for (int i = 0; i < n; ++i) acc = ts::ts_add4_rn(acc, ts::dbl_bits(d[i]));
  return ts::bits_dbl(acc);
}

// RN(s / n) through ts_div_int_rn.
extern "C" double host_div_int(double s, uint32_t n) { return ts::bits_dbl(ts::ts_div_int_rn(ts::dbl_bits(s), n)); }

// One addition through ts_add_rn.
extern "C" double host_add_rn(double a, double b) { return ts::bits_dbl(ts::ts_add_rn(ts::dbl_bits(a), ts::dbl_bits(b))); }

// Fast weight: returns 1 and the weight when the double-f32 path decides.
extern "C" int host_weight_ff(double d, double mean, float *w) { return ts::ts_weight_ff(d, mean, kTabFF, *w) ? 1 : 0; }

// The exact weight: (f32) exp(-(d / mean)).
extern "C" float host_weight_exact(double d, double mean) {
  return (float)ts::ts_exp64(-1.0 * (d / mean), kTab);
}

// The distance units * 2^qe as a double (ts_units_bits).
extern "C" double host_units_dbl(uint64_t units, int32_t qe) { return ts::bits_dbl(ts::ts_units_bits(units, qe)); }

