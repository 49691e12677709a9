// One-step ("plain") kernels and small helpers: medium preparation, the
// receiver gather / residual scatter, the imaging condition, the residual and
// misfit, the chain rule, and 16-bit checkpoint (de)quantisation.

#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "fdtd_internal.h"

namespace fdtd {
namespace {

__device__ __forceinline__ float operand(const StepArgs& a, const float* u, int y, int x) {
  if (y < 0 || y >= a.ny || x < 0 || x >= a.nx) return 0.f;
  const long long i = (long long)y * a.pitch + x;
  const float v = u[i];
  return a.adjoint == 1 ? __fmul_rn(a.coef[i], v) : v;
}

// D(b, u) = ((b_r (u_r - u) - b_l (u - u_l)) / dx^2 + (b_t (u_t - u) - b_b (u - u_b)) / dy^2:
// the conservative operator of 1DWaveSimulation.py:116-143 in 2-D.
__device__ __forceinline__ float dens_op(float c, float l, float r, float d, float t, float bl, float br, float bb,
                                         float bt, float idx2, float idy2) {
  const float fx = __fsub_rn(__fmul_rn(br, __fsub_rn(r, c)), __fmul_rn(bl, __fsub_rn(c, l)));
  const float fy = __fsub_rn(__fmul_rn(bt, __fsub_rn(t, c)), __fmul_rn(bb, __fsub_rn(c, d)));
  return __fmaf_rn(fy, idy2, __fmul_rn(fx, idx2));
}

__device__ __forceinline__ float dens_operand(const StepArgs& a, const float* u, int y, int x) {
  if (y < 0 || y >= a.ny || x < 0 || x >= a.nx) return 0.f;
  const long long i = (long long)y * a.pitch + x;
  return a.adjoint == 1 ? __fmul_rn(a.kap[i], u[i]) : u[i];
}

// Interior update of node (y, x) of shot s, sources included, before Mur.
__device__ float cell_next(const StepArgs& a, int s, int y, int x) {
  const long long plane = (long long)a.ny * a.pitch;
  const float* u = a.u + s * plane;
  const float* uo = a.u_old + s * plane;
  const long long i = (long long)y * a.pitch + x;
  if (a.kap) {
    // variable density: u+ = 2u - u- + kap D(b, u); the adjoint (1): l+ = 2l - l- + D(b, kap l)
    const long long bxs = a.pitch + 4;
    const float D = dens_op(dens_operand(a, u, y, x), dens_operand(a, u, y, x - 1), dens_operand(a, u, y, x + 1),
                            dens_operand(a, u, y - 1, x), dens_operand(a, u, y + 1, x), a.bx[y * bxs + x],
                            a.bx[y * bxs + x + 1], a.by[i], a.by[i + a.pitch], a.idx2, a.idy2);
    float un = a.adjoint == 1 ? leap_adj(u[i], uo[i], D) : leap(u[i], uo[i], a.kap[i], D);
    if (a.src_per_shot > 0) {
      float acc = 0.f;
      bool hit = false;
      for (int j = 0; j < a.src_per_shot; ++j) {
        const int e = s * a.src_per_shot + j;
        if (a.src_row[e] == y && a.src_col[e] == x && a.src_wave[e] >= 0) {
          const float v = (a.step < a.wave_len) ? a.waveforms[(long long)a.src_wave[e] * a.wave_len + a.step] : 0.f;
          acc = inj_acc(acc, a.src_w[e], v);
          hit = true;
        }
      }
      if (hit) un = inj_add(un, acc);
    }
    if (a.dense) un = inj_add(un, a.dense[s * plane + i]);
    return un;
  }
  const float nb = nbrq(operand(a, u, y, x - 1), operand(a, u, y, x + 1), operand(a, u, y - 1, x),
                        operand(a, u, y + 1, x), a.ratio);
  const float lap = __fmaf_rn(operand(a, u, y, x), a.qdiag, nb);  // Q = dy^2 lap
  // adjoint 1: l+ = 2l - l- + Q(coef l); adjoint 2 (w = coef l): the forward form
  float un = a.adjoint == 1 ? leap_adj(u[i], uo[i], lap) : leap(u[i], uo[i], a.coef[i], lap);
  if (a.src_per_shot > 0) {
    float acc = 0.f;
    bool hit = false;
    for (int j = 0; j < a.src_per_shot; ++j) {
      const int e = s * a.src_per_shot + j;
      if (a.src_row[e] == y && a.src_col[e] == x && a.src_wave[e] >= 0) {
        const float v = (a.step < a.wave_len)
                            ? a.waveforms[(long long)a.src_wave[e] * a.wave_len + a.step]
                            : 0.f;
        acc = inj_acc(acc, a.src_w[e], v);
        hit = true;
      }
    }
    if (hit) un = inj_add(un, acc);
  }
  if (a.dense) {
    const float d = a.dense[s * plane + i];
    un = inj_add(un, a.adjoint == 2 ? __fmul_rn(a.coef[i], d) : d);
  }
  return un;
}

__global__ void step_kernel(const StepArgs a) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int s = blockIdx.z;
  if (x >= a.nx || y >= a.ny) return;
  const long long plane = (long long)a.ny * a.pitch;
  const float* u = a.u + s * plane;
  const int ny = a.ny, nx = a.nx, P = a.pitch;
  const float* kl = a.mur;
  const float* kr = kl + ny;
  const float* kb = kr + ny;
  const float* kt = kb + nx;
  const float* ckx = kt + nx;
  const float* cky = ckx + 4;
  const bool bot = y == 0, top = y == ny - 1, lef = x == 0, rig = x == nx - 1;
  // ratios coef_edge / coef_inner for the w-form adjoint (1 otherwise)
  const float* rw = a.mur + 2 * ny + 2 * nx + 8;
  const bool wf = a.adjoint == 2;
  auto R = [&](const float* arr, int j) { return wf ? arr[j] : 1.0f; };
  const float* rl = rw;
  const float* rr = rl + ny;
  const float* rb = rr + ny;
  const float* rt = rb + nx;
  const float* crx = rt + nx;
  const float* cry = crx + 4;
  float out;
  if (!(bot || top || lef || rig)) {
    out = cell_next(a, s, y, x);
  } else if (!(lef || rig)) {  // row 0 or ny-1 (fdtd2d/torch_backend.py:218-223)
    const int yi = bot ? 1 : ny - 2;
    out = murw(R(bot ? rb : rt, x), u[yi * P + x], bot ? kb[x] : kt[x], cell_next(a, s, yi, x),
               u[y * P + x]);
  } else if (!(bot || top)) {  // column 0 or nx-1 (fdtd2d/torch_backend.py:212-217)
    const int xi = lef ? 1 : nx - 2;
    out = murw(R(lef ? rl : rr, y), u[y * P + xi], lef ? kl[y] : kr[y], cell_next(a, s, y, xi),
               u[y * P + x]);
  } else {  // corner from the updated edges (fdtd2d/torch_backend.py:225-232)
    const int ci = (bot ? 0 : 2) + (lef ? 0 : 1);
    const int yi = bot ? 1 : ny - 2, xi = lef ? 1 : nx - 2;
    const float inner = cell_next(a, s, yi, xi);
    const float ex = murw(R(bot ? rb : rt, xi), u[yi * P + xi], bot ? kb[xi] : kt[xi], inner, u[y * P + xi]);
    const float ey = murw(R(lef ? rl : rr, yi), u[yi * P + xi], lef ? kl[yi] : kr[yi], inner, u[yi * P + x]);
    const float fx = murw(R(crx, ci), u[y * P + xi], ckx[ci], ex, u[y * P + x]);
    const float fy = murw(R(cry, ci), u[yi * P + x], cky[ci], ey, u[y * P + x]);
    out = corner_avg(fx, fy);
  }
  a.u_next[s * plane + (long long)y * P + x] = out;
}

// One step of a PML grid: cell (y, x) of shot s. The face values on the cell's
// right and top faces are recomputed from the neighbours' old face fields (the
// same arithmetic the neighbour does for its own faces), so every value equals
// the fused kernel's. Beyond the grid u and psi are zero (the rigid wall behind
// the layer).
__global__ void step_pml_kernel(const StepArgs a, const float* __restrict__ pml,
                                const float* __restrict__ psx, const float* __restrict__ psy, float* psxn,
                                float* psyn) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int s = blockIdx.z;
  if (x >= a.nx || y >= a.ny) return;
  const int ny = a.ny, nx = a.nx, P = a.pitch;
  const long long plane = (long long)ny * P;
  const float* u = a.u + s * plane;
  const float* px = psx + s * plane;
  const float* py = psy + s * plane;
  auto U = [&](int yy, int xx) { return (yy < 0 || yy >= ny || xx < 0 || xx >= nx) ? 0.f : u[(long long)yy * P + xx]; };
  const float* sxc = pml;
  const float* sxf = pml + nx;
  const float* axf = pml + 2 * nx;
  const float* bxf = pml + 3 * nx;
  const float* syc = pml + PML_TABLES * nx;
  const float* syf = syc + ny;
  const float* ayf = syf + ny;
  const float* byf = ayf + ny;
  const long long i = (long long)y * P + x;
  const float uc = U(y, x), ul = U(y, x - 1), ur = U(y, x + 1), ud = U(y - 1, x), uu = U(y + 1, x);
  const float lap = __fmaf_rn(uc, a.qdiag, nbrq(ul, ur, ud, uu, a.ratio));  // Q = dy^2 lap
  const float pxl = pml_face(axf[x], px[i], syc[y], sxf[x], bxf[x], __fsub_rn(uc, ul));
  const float pxr = (x + 1 < nx) ? pml_face(axf[x + 1], px[i + 1], syc[y], sxf[x + 1], bxf[x + 1], __fsub_rn(ur, uc)) : 0.f;
  const float pyb = pml_face(ayf[y], py[i], sxc[x], syf[y], byf[y], __fsub_rn(uc, ud));
  const float pyt = (y + 1 < ny) ? pml_face(ayf[y + 1], py[i + P], sxc[x], syf[y + 1], byf[y + 1], __fsub_rn(uu, uc)) : 0.f;
  float A, M;
  pml_factors(sxc[x], syc[y], A, M);
  float un = pml_leap(uc, a.u_old[s * plane + i], a.coef[i], A, M, lap, pml_div(pxl, pxr, pyb, pyt));
  if (a.src_per_shot > 0) {
    float acc = 0.f;
    bool hit = false;
    for (int j = 0; j < a.src_per_shot; ++j) {
      const int e = s * a.src_per_shot + j;
      if (a.src_row[e] == y && a.src_col[e] == x && a.src_wave[e] >= 0) {
        const float v = (a.step < a.wave_len) ? a.waveforms[(long long)a.src_wave[e] * a.wave_len + a.step] : 0.f;
        acc = inj_acc(acc, a.src_w[e], v);
        hit = true;
      }
    }
    if (hit) un = inj_add(un, acc);
  }
  if (a.dense) {
    const float d = a.dense[s * plane + i];
    un = inj_add(un, a.adjoint == 2 ? __fmul_rn(a.coef[i], d) : d);
  }
  a.u_next[s * plane + i] = un;
  psxn[s * plane + i] = pxl;
  psyn[s * plane + i] = pyb;
}

// PML tables and the scaled coefficients of a padded medium, in one block: the
// largest speed (for sigma_max), then per column / row sigma at the centre and at
// the low face with the face decay and forcing scale (times dy^2), then
// coef = q (c dt / dy)^2.
__device__ __forceinline__ double pml_sigma(double xc, int n, int cells, double smax) {
  const double lo = (cells - 0.5) - xc, hi = xc - (n - cells - 0.5);
  double d = lo > hi ? lo : hi;
  if (d < 0.0) d = 0.0;
  const double r = d / cells;
  return smax * r * r;
}

__global__ void pml_prepare_kernel(const double* c, int ny, int nx, int pitch, double dt, double dx, double dy,
                                   int cells, double reflection, float* coef, float* pml) {
  __shared__ double red[32];
  double m = 0.0;
  for (long long i = threadIdx.x; i < (long long)ny * nx; i += blockDim.x) m = fmax(m, c[i]);
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_down_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x < 32) {
    m = (threadIdx.x < blockDim.x / 32) ? red[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_down_sync(0xffffffffu, m, o));
    if (threadIdx.x == 0) red[0] = m;
  }
  __syncthreads();
  const double cmax = red[0];
  const double smx = 3.0 * cmax * log(1.0 / reflection) / (2.0 * cells * dx);
  const double smy = 3.0 * cmax * log(1.0 / reflection) / (2.0 * cells * dy);
  float* col = pml;
  float* row = pml + PML_TABLES * nx;
  for (int i = threadIdx.x; i < nx; i += blockDim.x) {
    const double sc = pml_sigma(i, nx, cells, smx), sf = pml_sigma(i - 0.5, nx, cells, smx);
    // sigmas times dt / 2, the forcing scale times 2 / dt (and dy^2, the units of Q)
    col[i] = (float)(0.5 * dt * sc);
    col[nx + i] = (float)(0.5 * dt * sf);
    col[2 * nx + i] = (float)((1.0 - 0.5 * dt * sf) / (1.0 + 0.5 * dt * sf));
    col[3 * nx + i] = (float)(2.0 * (dy * dy) / (dx * dx * (1.0 + 0.5 * dt * sf)));
  }
  for (int j = threadIdx.x; j < ny; j += blockDim.x) {
    const double sc = pml_sigma(j, ny, cells, smy), sf = pml_sigma(j - 0.5, ny, cells, smy);
    row[j] = (float)(0.5 * dt * sc);
    row[ny + j] = (float)(0.5 * dt * sf);
    row[2 * ny + j] = (float)((1.0 - 0.5 * dt * sf) / (1.0 + 0.5 * dt * sf));
    row[3 * ny + j] = (float)(2.0 / (1.0 + 0.5 * dt * sf));  // (dt / dy^2) dy^2 times 2 / dt
  }
  for (long long k = threadIdx.x; k < (long long)ny * nx; k += blockDim.x) {
    const int y = (int)(k / nx), x = (int)(k - (long long)y * nx);
    const double q = 1.0 / (1.0 + 0.5 * dt * (pml_sigma(x, nx, cells, smx) + pml_sigma(y, ny, cells, smy)));
    const double cd = c[k] * dt / dy;
    coef[(long long)y * pitch + x] = (float)(cd * cd * q);
  }
}

// kappa = rho c^2 dt^2 (ny, pitch) and the face coefficients 1/rho = 2 / (rho_a +
// rho_b), an outer face taking its edge cell's rho: bx (ny, pitch + 4), by (ny + 1, pitch).
__global__ void density_prepare_kernel(const double* c, const double* rho, int ny, int nx, int pitch, double dt,
                                       float* kap, float* bx, float* by) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (y < ny && x < pitch) {
    float v = 0.f;
    if (x < nx) {
      const double cc = c[(long long)y * nx + x];
      v = (float)(dt * dt * rho[(long long)y * nx + x] * cc * cc);
    }
    kap[(long long)y * pitch + x] = v;
  }
  if (y < ny && x < pitch + 4) {
    float v = 0.f;
    if (x <= nx) {
      const int xa = x > 0 ? x - 1 : 0, xb = x < nx ? x : nx - 1;
      v = (float)(2.0 / (rho[(long long)y * nx + xa] + rho[(long long)y * nx + xb]));
    }
    bx[(long long)y * (pitch + 4) + x] = v;
  }
  if (y <= ny && x < pitch) {
    float v = 0.f;
    if (x < nx) {
      const int ya = y > 0 ? y - 1 : 0, yb = y < ny ? y : ny - 1;
      v = (float)(2.0 / (rho[(long long)ya * nx + x] + rho[(long long)yb * nx + x]));
    }
    by[(long long)y * pitch + x] = v;
  }
}

// One variable-density step's imaging (see image_density_launch): thread (y, x)
// owns cell (y, x), the x-face to its left (x = 0..nx) and the y-face below it
// (y = 0..ny), and sums the shots itself (no atomics).
__global__ void image_density_kernel(int ny, int nx, int pitch, float idx2, float idy2, int n_shots,
                                     const float* __restrict__ adj, const float* __restrict__ fwd,
                                     const float* __restrict__ kap, const float* __restrict__ bx,
                                     const float* __restrict__ by, double scale, double dt2, double* gk,
                                     double* gbx, double* gby) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const long long plane = (long long)ny * pitch, bxs = pitch + 4;
  auto F = [&](const float* f, int yy, int xx) {
    return (yy < 0 || yy >= ny || xx < 0 || xx >= nx) ? 0.f : f[(long long)yy * pitch + xx];
  };
  auto K = [&](int yy, int xx) {  // kappa without dt^2, float64
    return (yy < 0 || yy >= ny || xx < 0 || xx >= nx) ? 0.0 : (double)kap[(long long)yy * pitch + xx] / dt2;
  };
  double sk = 0.0, sx = 0.0, sy = 0.0;
  for (int s = 0; s < n_shots; ++s) {
    const float* w = adj + s * plane;
    const float* u = fwd + s * plane;
    if (y < ny && x < nx) {
      const long long i = (long long)y * pitch + x;
      const float D = dens_op(u[i], F(u, y, x - 1), F(u, y, x + 1), F(u, y - 1, x), F(u, y + 1, x), bx[y * bxs + x],
                              bx[y * bxs + x + 1], by[i], by[i + pitch], idx2, idy2);
      sk += (double)w[i] * (double)D;
    }
    if (y < ny && x <= nx)
      sx += (K(y, x - 1) * F(w, y, x - 1) - K(y, x) * F(w, y, x)) * ((double)F(u, y, x) - F(u, y, x - 1));
    if (y <= ny && x < nx)
      sy += (K(y - 1, x) * F(w, y - 1, x) - K(y, x) * F(w, y, x)) * ((double)F(u, y, x) - F(u, y - 1, x));
  }
  if (y < ny && x < nx) gk[(long long)y * pitch + x] += scale * sk;
  if (y < ny && x <= nx) gbx[(long long)y * bxs + x] += scale * sx * (double)idx2;
  if (y <= ny && x < nx) gby[(long long)y * pitch + x] += scale * sy * (double)idy2;
}

// g_m = -g_kappa rho / m^2 and g_rho = g_kappa / m + the face terms (db/drho = -b^2 / 2
// on an interior face, -b^2 on an outer one), zero off the mask.
__global__ void density_chain_kernel(int ny, int nx, int pitch, const double* m, const double* rho,
                                     const double* gk, const double* gbx, const double* gby, const uint8_t* mask,
                                     double* g_m, double* g_rho) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= nx || y >= ny) return;
  const long long i = (long long)y * nx + x, bxs = pitch + 4;
  auto R = [&](int yy, int xx) { return rho[(long long)yy * nx + xx]; };
  auto face = [](double ra, double rb) { const double b = 2.0 / (ra + rb); return b * b; };
  const double mi = m[i], ri = R(y, x);
  const double g = gk[(long long)y * pitch + x];
  double gr = g / mi;
  const double hl = -0.5 * gbx[y * bxs + x] * face(x > 0 ? R(y, x - 1) : ri, ri);
  const double hr = -0.5 * gbx[y * bxs + x + 1] * face(ri, x + 1 < nx ? R(y, x + 1) : ri);
  const double hb = -0.5 * gby[(long long)y * pitch + x] * face(y > 0 ? R(y - 1, x) : ri, ri);
  const double ht = -0.5 * gby[(long long)(y + 1) * pitch + x] * face(ri, y + 1 < ny ? R(y + 1, x) : ri);
  gr += (x == 0 ? 2.0 : 1.0) * hl + (x == nx - 1 ? 2.0 : 1.0) * hr + (y == 0 ? 2.0 : 1.0) * hb +
        (y == ny - 1 ? 2.0 : 1.0) * ht;
  const bool in = !mask || mask[i];
  g_m[i] = in ? -g * ri / (mi * mi) : 0.0;
  g_rho[i] = in ? gr : 0.0;
}

__global__ void gather_kernel(int pitch, long long plane, int n_shots, const float* f, int n_rx,
                              const int32_t* rc, const float* w, float* out,
                              long long shot_stride, long long rx_stride) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  const int s = blockIdx.y;
  if (r >= n_rx || s >= n_shots) return;
  const int r0 = rc[2 * r], c0 = rc[2 * r + 1];
  const float* fs = f + s * plane + (long long)r0 * pitch + c0;
  out[s * shot_stride + r * rx_stride] =
      gather4(fs[0], fs[1], fs[pitch], fs[pitch + 1], w[4 * r], w[4 * r + 1], w[4 * r + 2], w[4 * r + 3]);
}

__global__ void scatter_kernel(int pitch, long long plane, int n_shots, int n_nodes,
                               const int32_t* nodes, const float* w, const float* res,
                               long long shot_stride, long long rx_stride, float* dense) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int s = blockIdx.y;
  if (i >= n_nodes || s >= n_shots) return;
  const int32_t* nd = nodes + (long long)i * (2 + TAP_C);
  float acc = 0.f;
#pragma unroll
  for (int q = 0; q < TAP_C; ++q) {
    const int rid = nd[2 + q];
    if (rid >= 0) acc = inj_acc(acc, w[(long long)i * TAP_C + q], res[s * shot_stride + rid * rx_stride]);
  }
  dense[s * plane + (long long)nd[0] * pitch + nd[1]] = acc;
}

__device__ __forceinline__ float at0(const float* f, int ny, int nx, int pitch, int y, int x) {
  return (y >= 0 && y < ny && x >= 0 && x < nx) ? f[(long long)y * pitch + x] : 0.f;
}

__global__ void image_kernel(int ny, int nx, int pitch, float idx2, float idy2, float cdiag,
                             int n_shots, const float* adj, const float* fwd, double scale,
                             const float* coef_div, double* g) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= nx || y >= ny) return;
  const long long plane = (long long)ny * pitch;
  float acc = 0.f;
  for (int s = 0; s < n_shots; ++s) {
    const float* f = fwd + s * plane;
    const float lap = lap5(at0(f, ny, nx, pitch, y, x), at0(f, ny, nx, pitch, y, x - 1),
                           at0(f, ny, nx, pitch, y, x + 1), at0(f, ny, nx, pitch, y - 1, x),
                           at0(f, ny, nx, pitch, y + 1, x), idx2, idy2, cdiag);
    acc = __fmaf_rn(adj[s * plane + (long long)y * pitch + x], lap, acc);
  }
  // adjoint carried as w = coef * l: divide once by coef
  const double a = coef_div ? (double)acc / (double)coef_div[(long long)y * pitch + x] : (double)acc;
  g[(long long)y * pitch + x] += a * scale;
}

// The fused adjoint's gradient: its float64 imaging sums of w Q (w = coef l), scaled
// and divided by coef once per pass.
__global__ void grad_divide_kernel(const double* graw, const float* coef, double scale, double* g, long long n) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float c = coef[i];
  if (c != 0.f) g[i] += scale * graw[i] / (double)c;
}

__device__ __forceinline__ double mur_k(double c, double dt, double h) {
  return (c * dt - h) / (c * dt + h);
}

// b = (c dt / dy)^2, rounded once from float64 (the update in units of 1/dy^2).
__global__ void coef_kernel(const double* c, int ny, int nx, int pitch, double dt, double dy, float* coef) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= pitch || y >= ny) return;
  float v = 0.f;
  if (x < nx) {
    const double cd = c[(long long)y * nx + x] * dt / dy;
    v = (float)(cd * cd);
  }
  coef[(long long)y * pitch + x] = v;
}

__device__ __forceinline__ float sq_ratio(double a, double b) { return (float)((a / b) * (a / b)); }

// Mur coefficients, then (same layout, offset mur_len) the coefficient ratios
// coef_edge / coef_inner = (c_edge / c_inner)^2 that the adjoint in w = coef * l
// form needs.
__global__ void mur_kernel(const double* c, int ny, int nx, double dt, double dx, double dy,
                           float* mur) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int len = 2 * ny + 2 * nx + 8;
  float* kl = mur;
  float* kr = kl + ny;
  float* kb = kr + ny;
  float* kt = kb + nx;
  float* ckx = kt + nx;
  float* cky = ckx + 4;
  float* rl = mur + len;
  float* rr = rl + ny;
  float* rb = rr + ny;
  float* rt = rb + nx;
  float* crx = rt + nx;
  float* cry = crx + 4;
  auto C = [&](int y, int x) { return c[(long long)y * nx + x]; };
  if (i < ny) {
    const bool in = i >= 1 && i <= ny - 2;
    kl[i] = in ? (float)mur_k(C(i, 0), dt, dx) : 0.f;
    kr[i] = in ? (float)mur_k(C(i, nx - 1), dt, dx) : 0.f;
    rl[i] = in ? sq_ratio(C(i, 0), C(i, 1)) : 0.f;
    rr[i] = in ? sq_ratio(C(i, nx - 1), C(i, nx - 2)) : 0.f;
  }
  if (i < nx) {
    const bool in = i >= 1 && i <= nx - 2;
    kb[i] = in ? (float)mur_k(C(0, i), dt, dy) : 0.f;
    kt[i] = in ? (float)mur_k(C(ny - 1, i), dt, dy) : 0.f;
    rb[i] = in ? sq_ratio(C(0, i), C(1, i)) : 0.f;
    rt[i] = in ? sq_ratio(C(ny - 1, i), C(ny - 2, i)) : 0.f;
  }
  if (i < 4) {
    const int r = (i < 2) ? 0 : ny - 1, ri = (i < 2) ? 1 : ny - 2;
    const int col = (i & 1) ? nx - 1 : 0, ci = (i & 1) ? nx - 2 : 1;
    const double cc = C(r, col);
    ckx[i] = (float)mur_k(cc, dt, dx);
    cky[i] = (float)mur_k(cc, dt, dy);
    crx[i] = sq_ratio(cc, C(r, ci));
    cry[i] = sq_ratio(cc, C(ri, col));
  }
}

__global__ void residual_kernel(long long total, long long per_shot, int n_steps,
                                const float* traces, const float* obs, long long obs_stride,
                                const int32_t* mute, float* res, double* misfit) {
  double acc = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const long long s = i / per_shot;
    const long long rem = i - s * per_shot;
    const int r = (int)(rem / n_steps);
    float v = __fsub_rn(traces[i], obs[s * obs_stride + rem]);
    if (mute && mute[s] == r) v = 0.f;
    res[i] = v;
    acc += (double)v * (double)v;
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  __shared__ double part[32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) part[wid] = acc;
  __syncthreads();
  if (wid == 0) {
    acc = (lane < (int)(blockDim.x >> 5)) ? part[lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if (lane == 0) atomicAdd(misfit, 0.5 * acc);
  }
}

__global__ void chain_kernel(long long n, const double* g, const double* m, const uint8_t* mask,
                             double* out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    out[i] = (mask && !mask[i]) ? 0.0 : -g[i] / (m[i] * m[i]);
  }
}

// The value a checkpoint slot stores: the field itself, or with `minus` set the
// difference field - minus (the leapfrog step u - u_old).
__device__ __forceinline__ float ckpt_value(const float* src, const float* minus, long long i) {
  return minus ? __fsub_rn(src[i], minus[i]) : src[i];
}

__global__ void amax_kernel(const float* src, const float* minus, long long per_shot, unsigned* amax) {
  const int s = blockIdx.y;
  float a = 0.f;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < per_shot;
       i += (long long)gridDim.x * blockDim.x) {
    a = fmaxf(a, fabsf(ckpt_value(src, minus, s * per_shot + i)));
  }
  for (int o = 16; o > 0; o >>= 1) a = fmaxf(a, __shfl_down_sync(0xffffffffu, a, o));
  if ((threadIdx.x & 31) == 0) atomicMax(amax + s, __float_as_uint(a));
}

// Power-of-two scale that maps the largest magnitude to at most 2^15.
__device__ __forceinline__ float pow2_scale(unsigned amax_bits) {
  const float a = __uint_as_float(amax_bits);
  if (!(a > 0.f) || !isfinite(a)) return 1.f;
  int e;
  frexpf(a, &e);  // a = f * 2^e, f in [0.5, 1)
  return ldexpf(1.f, e - 15);
}

__global__ void quant_kernel(const float* src, const float* minus, void* dst, const unsigned* amax, float* scales,
                             long long per_shot, int store) {
  const int s = blockIdx.y;
  const float sc = pow2_scale(amax[s]);
  if (blockIdx.x == 0 && threadIdx.x == 0) scales[s] = sc;
  const float inv = 1.f / sc;  // exact: sc is a power of two
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < per_shot;
       i += (long long)gridDim.x * blockDim.x) {
    const float v = ckpt_value(src, minus, s * per_shot + i) * inv;
    if (store == 1) {
      reinterpret_cast<__half*>(dst)[s * per_shot + i] = __float2half_rn(v);
    } else {
      reinterpret_cast<__nv_bfloat16*>(dst)[s * per_shot + i] = __float2bfloat16_rn(v);
    }
  }
}

// dst = q * scale, or with `base` set dst = base - q * scale (u_old from u and u - u_old).
__global__ void dequant_kernel(const void* src, const float* scales, const float* base, float* dst,
                               long long per_shot, int store) {
  const int s = blockIdx.y;
  const float sc = scales[s];
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < per_shot;
       i += (long long)gridDim.x * blockDim.x) {
    const long long k = s * per_shot + i;
    const float q = (store == 1) ? __half2float(reinterpret_cast<const __half*>(src)[k])
                                 : __bfloat162float(reinterpret_cast<const __nv_bfloat16*>(src)[k]);
    const float v = q * sc;  // exact: sc is a power of two
    dst[k] = base ? __fsub_rn(base[k], v) : v;
  }
}

}  // namespace

cudaError_t step_launch(const StepArgs& a, cudaStream_t st) {
  dim3 block(32, 8);
  dim3 grid((a.nx + 31) / 32, (a.ny + 7) / 8, a.n_shots);
  step_kernel<<<grid, block, 0, st>>>(a);
  return cudaGetLastError();
}

cudaError_t gather_launch(int ny, int pitch, int n_shots, const float* fields, int n_rx,
                          const int32_t* rx_rc, const float* rx_w, float* out,
                          long long shot_stride, long long rx_stride, cudaStream_t st) {
  dim3 grid((n_rx + 127) / 128, n_shots);
  gather_kernel<<<grid, 128, 0, st>>>(pitch, (long long)ny * pitch, n_shots, fields, n_rx, rx_rc,
                                      rx_w, out, shot_stride, rx_stride);
  return cudaGetLastError();
}

cudaError_t scatter_launch(int ny, int pitch, int n_shots, int n_nodes, const int32_t* nodes,
                           const float* w, const float* res, long long shot_stride,
                           long long rx_stride, float* dense, cudaStream_t st) {
  dim3 grid((n_nodes + 127) / 128, n_shots);
  scatter_kernel<<<grid, 128, 0, st>>>(pitch, (long long)ny * pitch, n_shots, n_nodes, nodes, w,
                                       res, shot_stride, rx_stride, dense);
  return cudaGetLastError();
}

cudaError_t grad_divide_launch(const double* graw, const float* coef, double scale, double* g, long long n,
                               cudaStream_t st) {
  const int threads = 256;
  const long long blocks = (n + threads - 1) / threads;
  grad_divide_kernel<<<(unsigned)blocks, threads, 0, st>>>(graw, coef, scale, g, n);
  return cudaGetLastError();
}

cudaError_t image_launch(int ny, int nx, int pitch, float idx2, float idy2, float cdiag,
                         int n_shots, const float* adj, const float* fwd, double scale,
                         const float* coef_div, double* g, cudaStream_t st) {
  dim3 block(32, 8);
  dim3 grid((nx + 31) / 32, (ny + 7) / 8);
  image_kernel<<<grid, block, 0, st>>>(ny, nx, pitch, idx2, idy2, cdiag, n_shots, adj, fwd,
                                       scale, coef_div, g);
  return cudaGetLastError();
}

cudaError_t prepare_medium_launch(const double* c, int ny, int nx, int pitch, double dt,
                                  double dx, double dy, float* coef, float* mur,
                                  cudaStream_t st) {
  dim3 block(32, 8);
  dim3 grid((pitch + 31) / 32, (ny + 7) / 8);
  coef_kernel<<<grid, block, 0, st>>>(c, ny, nx, pitch, dt, dy, coef);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  const int n = (ny > nx ? ny : nx);
  mur_kernel<<<(n + 255) / 256, 256, 0, st>>>(c, ny, nx, dt, dx, dy, mur);
  return cudaGetLastError();
}

cudaError_t step_pml_launch(const StepArgs& a, const float* pml, const float* psx,
                            const float* psy, float* psx_next, float* psy_next, cudaStream_t st) {
  dim3 block(32, 8);
  dim3 grid((a.nx + 31) / 32, (a.ny + 7) / 8, a.n_shots);
  step_pml_kernel<<<grid, block, 0, st>>>(a, pml, psx, psy, psx_next, psy_next);
  return cudaGetLastError();
}

cudaError_t prepare_pml_launch(const double* c, int ny, int nx, int pitch, double dt, double dx, double dy,
                               int cells, double reflection, float* coef, float* pml, cudaStream_t st) {
  pml_prepare_kernel<<<1, 1024, 0, st>>>(c, ny, nx, pitch, dt, dx, dy, cells, reflection, coef, pml);
  return cudaGetLastError();
}

cudaError_t prepare_density_launch(const double* c, const double* rho, int ny, int nx, int pitch, double dt,
                                   double dx, double dy, float* kap, float* bx, float* by, float* mur,
                                   cudaStream_t st) {
  dim3 block(32, 8);
  dim3 grid((pitch + 4 + 31) / 32, (ny + 1 + 7) / 8);
  density_prepare_kernel<<<grid, block, 0, st>>>(c, rho, ny, nx, pitch, dt, kap, bx, by);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  const int n = (ny > nx ? ny : nx);
  mur_kernel<<<(n + 255) / 256, 256, 0, st>>>(c, ny, nx, dt, dx, dy, mur);
  return cudaGetLastError();
}

cudaError_t image_density_launch(int ny, int nx, int pitch, float idx2, float idy2, int n_shots, const float* adj,
                                 const float* fwd, const float* kap, const float* bx, const float* by, double scale,
                                 double dt2, double* gk, double* gbx, double* gby, cudaStream_t st) {
  dim3 block(32, 8);
  dim3 grid((nx + 1 + 31) / 32, (ny + 1 + 7) / 8);
  image_density_kernel<<<grid, block, 0, st>>>(ny, nx, pitch, idx2, idy2, n_shots, adj, fwd, kap, bx, by, scale,
                                               dt2, gk, gbx, gby);
  return cudaGetLastError();
}

cudaError_t density_chain_launch(int ny, int nx, int pitch, const double* m, const double* rho,
                                 const double* gk, const double* gbx, const double* gby, const uint8_t* mask,
                                 double* g_m, double* g_rho, cudaStream_t st) {
  dim3 block(32, 8);
  dim3 grid((nx + 31) / 32, (ny + 7) / 8);
  density_chain_kernel<<<grid, block, 0, st>>>(ny, nx, pitch, m, rho, gk, gbx, gby, mask, g_m, g_rho);
  return cudaGetLastError();
}

cudaError_t residual_launch(int n_shots, int n_rx, int n_steps, const float* traces,
                            const float* observed, long long obs_shot_stride,
                            const int32_t* mute, float* residual, double* misfit,
                            cudaStream_t st) {
  const long long per_shot = (long long)n_rx * n_steps;
  const long long total = per_shot * n_shots;
  long long blocks = (total + 255) / 256;
  if (blocks > 4096) blocks = 4096;
  if (blocks < 1) blocks = 1;
  residual_kernel<<<(int)blocks, 256, 0, st>>>(total, per_shot, n_steps, traces, observed,
                                               obs_shot_stride, mute, residual, misfit);
  return cudaGetLastError();
}

cudaError_t chain_rule_launch(long long n, const double* g, const double* m,
                              const uint8_t* mask, double* out, cudaStream_t st) {
  long long blocks = (n + 255) / 256;
  if (blocks > 4096) blocks = 4096;
  if (blocks < 1) blocks = 1;
  chain_kernel<<<(int)blocks, 256, 0, st>>>(n, g, m, mask, out);
  return cudaGetLastError();
}

cudaError_t quantize_launch(const float* src, const float* minus, void* dst, float* scales, int n_shots,
                            long long per_shot, int store, cudaStream_t st) {
  // scales holds 2 * n_shots floats: [0, n) amax scratch, [n, 2n) the scales.
  unsigned* amax = reinterpret_cast<unsigned*>(scales);
  cudaError_t e = cudaMemsetAsync(amax, 0, sizeof(unsigned) * n_shots, st);
  if (e != cudaSuccess) return e;
  dim3 grid(64, n_shots);
  amax_kernel<<<grid, 256, 0, st>>>(src, minus, per_shot, amax);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  quant_kernel<<<grid, 256, 0, st>>>(src, minus, dst, amax, scales + n_shots, per_shot, store);
  return cudaGetLastError();
}

cudaError_t dequantize_launch(const void* src, const float* scales, const float* base, float* dst, int n_shots,
                              long long per_shot, int store, cudaStream_t st) {
  dim3 grid(64, n_shots);
  dequant_kernel<<<grid, 256, 0, st>>>(src, scales + n_shots, base, dst, per_shot, store);
  return cudaGetLastError();
}

}  // namespace fdtd
