// aph_diag.cu -- device evaluation of the exact-mode integer-pipe operations (aph_math.cuh),
// so that tests can compare them bit for bit with the IEEE operations they replace.
#include "../../include/aph_hydro.h"
#include "aph_capi_internal.h"
#define APH_EXACT 1
#include "aph_math.cuh"

using namespace aph;

namespace {

__global__ void k_exact_ops(int op, const double *x, double *out, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const double v = x[i];
    double r;
    if (op == 0) r = div6_x(v);
    else if (op == 1) r = half_x(v);
    else if (op == 2) r = twice_x(v);
    else r = tame(v) ? 1.0 : 0.0;
    out[i] = r;
  }
}

__global__ void k_exact_ops2(int op, const double *x, const double *y, double *out, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const double a = x[i], b = y[i];
    double r;
    if (op == 0) r = add_x(a, b);
    else if (op == 1) r = sub_x(a, b);
    else if (op == 2) r = mulk_x<3, 0>(a);
    else if (op == 3) r = mulk_x<3, 1>(a);
    else if (op == 4) r = mulk_x<5, -2>(a);
    else if (op == 5) r = a / b;
    else if (op == 6) r = __drcp_rn(b);
    else if (op == 7) r = sqrt(a);
    else r = div_rcp(a, b, __drcp_rn(b));
    out[i] = r;
  }
}

}  // namespace

extern "C" aph_status aph_diag_exact_ops2(int op, const double *x, const double *y, double *out,
                                          long long n, void *stream) {
  clear_error();
  if (op < 0 || op > 8) return fail(APH_ERR_INVALID, "op %d not in 0..8", op);
  if (n < 0 || (n > 0 && (!x || !y || !out))) return fail(APH_ERR_INVALID, "NULL argument");
  if (n == 0) return APH_OK;
  const long long blocks = (n + 255) / 256;
  k_exact_ops2<<<(unsigned)(blocks < 152 * 16 ? blocks : 152 * 16), 256, 0, (cudaStream_t)stream>>>(
      op, x, y, out, n);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? APH_OK : cuda_fail(e, "diag_exact_ops2");
}

extern "C" aph_status aph_diag_exact_ops(int op, const double *x, double *out, long long n,
                                         void *stream) {
  clear_error();
  if (op < 0 || op > 3) return fail(APH_ERR_INVALID, "op %d not in 0..3", op);
  if (n < 0 || (n > 0 && (!x || !out))) return fail(APH_ERR_INVALID, "NULL argument");
  if (n == 0) return APH_OK;
  const long long blocks = (n + 255) / 256;
  k_exact_ops<<<(unsigned)(blocks < 152 * 16 ? blocks : 152 * 16), 256, 0, (cudaStream_t)stream>>>(
      op, x, out, n);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? APH_OK : cuda_fail(e, "diag_exact_ops");
}
