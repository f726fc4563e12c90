// Host build of the weight primitives of ts_common.h, for the CPU tests.
#include "ts_common.h"

static const double kTab[64] = {TS_EXP2_TABLE_VALUES};
static const float kTabFF[128] = {TS_EXP2_FF_TABLE_VALUES};

extern "C" double host_exp(double x) { return ts::ts_exp64(x, kTab); }
extern "C" double host_div(double a, double b) { return ts::ts_div_markstein(a, b, 1.0 / b); }

// Fast weight: returns 1 and the weight when the double-f32 path decides.
extern "C" int host_weight_ff(double d, double mean, float *w) { return ts::ts_weight_ff(d, mean, kTabFF, *w) ? 1 : 0; }

// The exact weight: (f32) exp(-(d / mean)).
extern "C" float host_weight_exact(double d, double mean) {
  return (float)ts::ts_exp64(-1.0 * (d / mean), kTab);
}
