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

// ---- bicubic transfer of m between grid levels (invert_ring.py:1048-1068)
//
// The reference calls torch.nn.functional.grid_sample(mode="bicubic",
// padding_mode="border", align_corners=True) in float64. Its bicubic is Keys'
// cubic convolution with a = -0.75 on the 4 x 4 neighbours of the source
// position, rows interpolated first along x, then the four results along y;
// each neighbour index is clamped into the grid (border padding).

constexpr double CUBIC_A = -0.75;

__device__ __forceinline__ double cubic_near(double x) {  // |x| <= 1
  return __dadd_rn(__dmul_rn(__dmul_rn(__dsub_rn(__dmul_rn(CUBIC_A + 2.0, x), CUBIC_A + 3.0), x), x), 1.0);
}

__device__ __forceinline__ double cubic_far(double x) {  // 1 < |x| < 2
  return __dsub_rn(
      __dmul_rn(__dadd_rn(__dmul_rn(__dsub_rn(__dmul_rn(CUBIC_A, x), 5.0 * CUBIC_A), x), 8.0 * CUBIC_A), x),
      4.0 * CUBIC_A);
}

__device__ __forceinline__ double cubic_1d(double v0, double v1, double v2, double v3, double t) {
  const double c0 = cubic_far(__dadd_rn(t, 1.0)), c1 = cubic_near(t);
  const double s = __dsub_rn(1.0, t);
  const double c2 = cubic_near(s), c3 = cubic_far(__dadd_rn(s, 1.0));
  return __dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(v0, c0), __dmul_rn(v1, c1)), __dmul_rn(v2, c2)), __dmul_rn(v3, c3));
}

__device__ __forceinline__ double tap(const double* src, int ny, int nx, long long iy, long long ix) {
  const long long y = iy < 0 ? 0 : (iy > ny - 1 ? ny - 1 : iy);
  const long long x = ix < 0 ? 0 : (ix > nx - 1 ? nx - 1 : ix);
  return src[y * nx + x];
}

__global__ void resize_kernel(const double* __restrict__ src, int sny, int snx, const double* __restrict__ sx,
                              const double* __restrict__ sy, double* __restrict__ dst, int tny, int tnx,
                              const double* __restrict__ tx, const double* __restrict__ ty, double background) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)tny * tnx) return;
  const int i = (int)(idx / tnx), j = (int)(idx - (long long)i * tnx);
  // normalised coordinates as the reference builds them on the host
  const double u = __dsub_rn(__ddiv_rn(__dmul_rn(2.0, __dsub_rn(tx[j], sx[0])), __dsub_rn(sx[snx - 1], sx[0])), 1.0);
  const double v = __dsub_rn(__ddiv_rn(__dmul_rn(2.0, __dsub_rn(ty[i], sy[0])), __dsub_rn(sy[sny - 1], sy[0])), 1.0);
  if (fabs(u) > 1.0 || fabs(v) > 1.0) {
    dst[idx] = background;
    return;
  }
  // align_corners = True: ((coord + 1) / 2) * (size - 1)
  const double fx = __dmul_rn(__ddiv_rn(__dadd_rn(u, 1.0), 2.0), (double)(snx - 1));
  const double fy = __dmul_rn(__ddiv_rn(__dadd_rn(v, 1.0), 2.0), (double)(sny - 1));
  const double x0 = floor(fx), y0 = floor(fy);
  const double tx_ = __dsub_rn(fx, x0), ty_ = __dsub_rn(fy, y0);
  const long long ix = (long long)x0, iy = (long long)y0;
  double rows[4];
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const long long yy = iy - 1 + r;
    rows[r] = cubic_1d(tap(src, sny, snx, yy, ix - 1), tap(src, sny, snx, yy, ix), tap(src, sny, snx, yy, ix + 1),
                       tap(src, sny, snx, yy, ix + 2), tx_);
  }
  dst[idx] = cubic_1d(rows[0], rows[1], rows[2], rows[3], ty_);
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

extern "C" int32_t fdtd_resize_slowness(const double* src, int32_t src_ny, int32_t src_nx, const double* src_x,
                                        const double* src_y, double* dst, int32_t dst_ny, int32_t dst_nx,
                                        const double* dst_x, const double* dst_y, double background,
                                        void* stream) {
  if (!src || !dst || !src_x || !src_y || !dst_x || !dst_y) return fail(FDTD_ERR_INVALID, "resize: null argument");
  if (src_ny < 2 || src_nx < 2 || dst_ny < 1 || dst_nx < 1) return fail(FDTD_ERR_INVALID, "resize: grids too small");
  const long long n = (long long)dst_ny * dst_nx;
  resize_kernel<<<blocks(n), BLOCK, 0, (cudaStream_t)stream>>>(src, src_ny, src_nx, src_x, src_y, dst, dst_ny,
                                                               dst_nx, dst_x, dst_y, background);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? FDTD_OK : cuda_fail(e, "resize launch");
}
