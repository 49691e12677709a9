// Device-side inversion helpers: the Tikhonov / total-variation regularisers on
// the slowness squared m, the box projection of m and one projected Adam step,
// all in float64 on (ny, nx) row-major arrays. They keep an FWI iteration on the
// device: the reference copies the float64 gradient to the host every iteration
// (invert_ring.py:657) and runs Adam in NumPy (invert_ring.py:817-861).
//
// Every expression keeps NumPy's operation order with explicit round-to-nearest
// intrinsics (no contraction into FMA), so element values match the host
// restatement bit for bit; only the reductions (values, norms) differ in order.

#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>

#include "../../include/fdtd_gb300.h"
#include "fdtd_internal.h"

namespace fdtd {
namespace {

constexpr int BLOCK = 256;

__device__ __forceinline__ bool in_mask(const uint8_t* mask, long long i) { return mask[i] != 0; }

// Forward difference along x at (i, j) when both cells lie in the mask, else 0
// (fdtd2d/inversion/misfit.py:28-33 and 55-56).
__device__ __forceinline__ double diff_x(const double* m, const uint8_t* mask, int nx, int i, int j) {
  if (j < 0 || j + 1 >= nx) return 0.0;
  const long long a = (long long)i * nx + j;
  return (in_mask(mask, a) && in_mask(mask, a + 1)) ? __dsub_rn(m[a + 1], m[a]) : 0.0;
}

__device__ __forceinline__ double diff_y(const double* m, const uint8_t* mask, int ny, int nx, int i, int j) {
  if (i < 0 || i + 1 >= ny) return 0.0;
  const long long a = (long long)i * nx + j;
  return (in_mask(mask, a) && in_mask(mask, a + nx)) ? __dsub_rn(m[a + nx], m[a]) : 0.0;
}

// sqrt(dx^2 + dy^2 + eps^2) in NumPy's order (misfit.py:57).
__device__ __forceinline__ double tv_norm(double dx, double dy, double eps) {
  return __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(eps, eps)));
}

__device__ __forceinline__ double block_sum(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) red[w] = v;
  __syncthreads();
  v = (threadIdx.x < blockDim.x / 32) ? red[threadIdx.x] : 0.0;
  if (w == 0)
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// grad += tikhonov_grad + tv_grad on the mask (zero elsewhere);
// value += 0.5 alpha sum(dm^2) + tv sum(norm - eps).
__global__ void reg_kernel(int ny, int nx, const double* __restrict__ m, const uint8_t* __restrict__ mask,
                           double alpha, double tv, double eps, double* __restrict__ grad, double* value) {
  __shared__ double red[BLOCK / 32];
  const long long n = (long long)ny * nx;
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double part = 0.0;
  if (idx < n) {
    const int i = (int)(idx / nx), j = (int)(idx - (long long)i * nx);
    double g_tik = 0.0, g_tv = 0.0;
    if (alpha > 0.0) {
      // misfit.py:19-44: g[:, 1:] += cx; g[:, :-1] -= cx; g[1:, :] += cy; g[:-1, :] -= cy
      const double dxm = diff_x(m, mask, nx, i, j), dym = diff_y(m, mask, ny, nx, i, j);
      const double cx_l = __dmul_rn(alpha, diff_x(m, mask, nx, i, j - 1));
      const double cy_d = __dmul_rn(alpha, diff_y(m, mask, ny, nx, i - 1, j));
      g_tik = __dsub_rn(__dadd_rn(__dsub_rn(cx_l, __dmul_rn(alpha, dxm)), cy_d), __dmul_rn(alpha, dym));
      part = __dadd_rn(part, __dmul_rn(__dmul_rn(0.5, alpha), __dadd_rn(__dmul_rn(dxm, dxm), __dmul_rn(dym, dym))));
    }
    if (tv > 0.0) {
      // misfit.py:47-71: g -= gx + gy; g[:, 1:] += gx[:, :-1]; g[1:, :] += gy[:-1, :]
      const double dx0 = diff_x(m, mask, nx, i, j), dy0 = diff_y(m, mask, ny, nx, i, j);
      const double n0 = tv_norm(dx0, dy0, eps);
      const double gx0 = __ddiv_rn(__dmul_rn(tv, dx0), n0), gy0 = __ddiv_rn(__dmul_rn(tv, dy0), n0);
      double gxl = 0.0, gyd = 0.0;
      if (j >= 1) {
        const double dxl = diff_x(m, mask, nx, i, j - 1), dyl = diff_y(m, mask, ny, nx, i, j - 1);
        gxl = __ddiv_rn(__dmul_rn(tv, dxl), tv_norm(dxl, dyl, eps));
      }
      if (i >= 1) {
        const double dxd = diff_x(m, mask, nx, i - 1, j), dyd = diff_y(m, mask, ny, nx, i - 1, j);
        gyd = __ddiv_rn(__dmul_rn(tv, dyd), tv_norm(dxd, dyd, eps));
      }
      g_tv = __dadd_rn(__dadd_rn(__dsub_rn(0.0, __dadd_rn(gx0, gy0)), gxl), gyd);
      part = __dadd_rn(part, __dmul_rn(tv, __dsub_rn(n0, eps)));
    }
    if (in_mask(mask, idx)) grad[idx] = __dadd_rn(grad[idx], __dadd_rn(g_tik, g_tv));
    else grad[idx] = 0.0;
  }
  const double s = block_sum(part, red);
  if (threadIdx.x == 0 && s != 0.0) atomicAdd(value, s);
}

// np.clip(m, lo, hi) with the exterior set to the background (invert_ring.py:559-565).
__device__ __forceinline__ double project1(double v, bool inside, double lo, double hi, double ext) {
  return inside ? fmin(fmax(v, lo), hi) : ext;
}

__global__ void project_kernel(long long n, double* m, const uint8_t* mask, double lo, double hi, double ext) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) m[i] = project1(m[i], in_mask(mask, i), lo, hi, ext);
}

// One projected Adam step (invert_ring.py:842-853) on the mask.
__global__ void adam_kernel(long long n, double* m, const double* __restrict__ g, const uint8_t* mask,
                           double* first, double* second, double lr, double beta1, double beta2,
                           double eps, double bc1, double bc2, double lo, double hi, double ext) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const bool inside = in_mask(mask, i);
  double v = m[i];
  if (inside) {
    const double gi = g[i];
    const double f = __dadd_rn(__dmul_rn(beta1, first[i]), __dmul_rn(__dsub_rn(1.0, beta1), gi));
    const double s = __dadd_rn(__dmul_rn(beta2, second[i]), __dmul_rn(__dsub_rn(1.0, beta2), __dmul_rn(gi, gi)));
    first[i] = f;
    second[i] = s;
    const double fh = __ddiv_rn(f, bc1), sh = __ddiv_rn(s, bc2);
    const double update = __ddiv_rn(__dmul_rn(lr, fh), __dadd_rn(__dsqrt_rn(sh), eps));
    v = __dsub_rn(v, update);
  }
  m[i] = project1(v, inside, lo, hi, ext);
}

int blocks(long long n) { return (int)((n + BLOCK - 1) / BLOCK); }

}  // namespace
}  // namespace fdtd

using namespace fdtd;

extern "C" int32_t fdtd_regularization(int32_t ny, int32_t nx, const double* m, const uint8_t* mask,
                                       double alpha, double tv, double tv_eps, double* grad, double* value,
                                       void* stream) {
  if (ny < 1 || nx < 1 || !m || !mask || !grad || !value) return fail(FDTD_ERR_INVALID, "regularization: bad argument");
  if (alpha < 0.0 || tv < 0.0) return fail(FDTD_ERR_INVALID, "regularization weights must be non-negative");
  if (tv > 0.0 && !(tv_eps > 0.0)) return fail(FDTD_ERR_INVALID, "total variation needs tv_eps > 0");
  const long long n = (long long)ny * nx;
  reg_kernel<<<blocks(n), BLOCK, 0, (cudaStream_t)stream>>>(ny, nx, m, mask, alpha, tv, tv_eps, grad, value);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? FDTD_OK : cuda_fail(e, "regularization launch");
}

extern "C" int32_t fdtd_project(int64_t n, double* m, const uint8_t* mask, double m_min, double m_max,
                                double m_exterior, void* stream) {
  if (n < 0 || !m || !mask) return fail(FDTD_ERR_INVALID, "project: bad argument");
  if (!(m_min <= m_max)) return fail(FDTD_ERR_INVALID, "project: m_min must not exceed m_max");
  if (n == 0) return FDTD_OK;
  project_kernel<<<blocks(n), BLOCK, 0, (cudaStream_t)stream>>>(n, m, mask, m_min, m_max, m_exterior);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? FDTD_OK : cuda_fail(e, "project launch");
}

extern "C" int32_t fdtd_adam_step(int64_t n, double* m, const double* grad, const uint8_t* mask, double* first,
                                  double* second, double learning_rate, double beta1, double beta2,
                                  double epsilon, int32_t iteration, double m_min, double m_max,
                                  double m_exterior, void* stream) {
  if (n < 0 || !m || !grad || !mask || !first || !second) return fail(FDTD_ERR_INVALID, "adam: bad argument");
  if (iteration < 1) return fail(FDTD_ERR_INVALID, "adam: iteration counts from 1");
  if (!(m_min <= m_max)) return fail(FDTD_ERR_INVALID, "adam: m_min must not exceed m_max");
  if (n == 0) return FDTD_OK;
  // bias corrections 1 - beta**t with the C library's pow, as Python evaluates them
  const double bc1 = 1.0 - std::pow(beta1, (double)iteration), bc2 = 1.0 - std::pow(beta2, (double)iteration);
  adam_kernel<<<blocks(n), BLOCK, 0, (cudaStream_t)stream>>>(n, m, grad, mask, first, second, learning_rate,
                                                             beta1, beta2, epsilon, bc1, bc2, m_min, m_max,
                                                             m_exterior);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? FDTD_OK : cuda_fail(e, "adam launch");
}
