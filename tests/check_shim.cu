// Host build of the true-residual check of the FP64 / double-float PCG
// (scalar_after_check in graphitethree_gb300/csrc/nlgb_core.cuh) for
// tests/test_true_residual_check.py: a plain C entry point over the same
// __host__ __device__ code the kernels run.
#include "nlgb_core.cuh"

#include <cstring>

using namespace nlgb;

extern "C" int shim_after_check(double thresh2, double rthresh2, double bnorm2, double rr, double rr_true,
                                int checks, int cont_ok, long long iter, long long max_iter, int precision,
                                int zero_rhs, int status, double* rthresh2_out, int* checks_out,
                                int* status_out) {
  SysState st;
  std::memset(&st, 0, sizeof(st));
  st.thresh2 = thresh2;
  st.rthresh2 = rthresh2;
  st.bnorm2 = bnorm2;
  st.rr = rr;
  st.rr_true = rr_true;
  st.checks = checks;
  st.cont_ok = cont_ok;
  st.iter = iter;
  st.max_iter = max_iter;
  st.precision = precision;
  st.zero_rhs = zero_rhs;
  st.status = status;
  const bool cont = scalar_after_check(&st);
  *rthresh2_out = st.rthresh2;
  *checks_out = st.checks;
  *status_out = st.status;
  return cont ? 1 : 0;
}
