// Host build of the double-float primitives (graphitethree_gb300/csrc/nlgb_df.cuh)
// for tests/test_df_arith.py: plain C entry points over the same inline code
// the kernels use.  Built with -ffp-contract=off (no FMA contraction).
#include "nlgb_df.cuh"

using namespace nlgb;

extern "C" {
void df_two_sum(float a, float b, float* out) { const float2 r = df::two_sum(a, b); out[0] = r.x; out[1] = r.y; }
void df_add(const float* a, const float* b, float* out) {
  const float2 r = df::dadd(df::make(a[0], a[1]), df::make(b[0], b[1])); out[0] = r.x; out[1] = r.y;
}
void df_mul(const float* a, const float* b, float* out) {
  const float2 r = df::dmul(df::make(a[0], a[1]), df::make(b[0], b[1])); out[0] = r.x; out[1] = r.y;
}
void df_mac(const float* acc, const float* a, const float* b, float* out) {
  const float2 r = df::mac(df::make(acc[0], acc[1]), df::make(a[0], a[1]), df::make(b[0], b[1]));
  out[0] = r.x; out[1] = r.y;
}
void df_from_double(double d, float* out) { const float2 r = df::from_double(d); out[0] = r.x; out[1] = r.y; }
double df_to_double(const float* a) { return df::to_double(df::make(a[0], a[1])); }
}
