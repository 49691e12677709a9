// Internal declarations shared by the translation units of the engine library.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/fdtd_gb300.h"
#include "fdtd_device.cuh"

namespace fdtd {

// Error state of the C ABI (per host thread).
void set_error(const std::string& msg);
int32_t fail(int32_t code, const std::string& msg);
int32_t cuda_fail(cudaError_t e, const char* what);

// Argument checks shared by the entry points (fdtd_plan.cpp): the grid's shape,
// spacings and medium pointers; for the plain per-shot forms also shots, steps,
// receivers inside the grid (their 2 x 2 footprint included) and every used
// source entry's node and waveform index.
int32_t validate_grid(const fdtd_grid& g);
int32_t validate_plain_problem(const fdtd_problem& prob);

// Temporally blocked kernel (fdtd_tb.cu).
cudaError_t tb_launch(const TbParams& p, int ky, int mode, int grid, size_t smem, cudaStream_t st);
// Shared memory the temporally blocked kernels may declare statically (reserved out
// of the 227 KB per CTA when a plan sizes its dynamic shared memory).
constexpr size_t TB_STATIC_SMEM = 64;
// Sets the dynamic shared-memory attribute of the kernel a launch would use (the
// PML family for pml).
cudaError_t tb_configure(int ky, int mode, int nwarps, size_t smem, bool pml);
// One launch over the items of several plans (same rows per lane and warps).
cudaError_t tb_group_launch(const TbGroup& g, int ky, int nwarps, int mode, bool adj_coef, int grid, size_t smem,
                            cudaStream_t st);
// Static shared memory of the grouped kernel (its copy of one plan's parameters).
size_t tb_group_static_smem();

// One-step kernels and helpers (fdtd_kernels.cu).
struct StepArgs {
  int ny, nx, pitch;
  float idx2, idy2, cdiag;
  float ratio, qdiag;  // the stencil Q = dy^2 lap (fdtd_device.cuh nbrq)
  const float* coef;   // b = (c dt / dy)^2
  const float* mur;
  int n_shots;
  const float* u_old;
  const float* u;
  float* u_next;
  int src_per_shot;
  const int32_t* src_row;
  const int32_t* src_col;
  const float* src_w;
  const int32_t* src_wave;
  const float* waveforms;
  int wave_len;
  int step;
  const float* dense;
  int adjoint;
  // variable density (kap != nullptr): rho c^2 dt^2 per cell and 1/rho on the
  // faces, bx (ny, pitch + 4) between columns x-1 and x, by (ny + 1, pitch)
  const float* kap = nullptr;
  const float* bx = nullptr;
  const float* by = nullptr;
};
cudaError_t step_launch(const StepArgs& a, cudaStream_t st);
// Variable density: kappa = rho c^2 dt^2, the face coefficients and the Mur table.
cudaError_t prepare_density_launch(const double* c, const double* rho, int ny, int nx, int pitch, double dt,
                                   double dx, double dy, float* kap, float* bx, float* by, float* mur,
                                   cudaStream_t st);
// Imaging of a variable-density step: g_kappa += scale sum_s adj D(b, fwd) per cell,
// and per face g_b += scale sum_s (adj_a kappa_a - adj_b kappa_b) (fwd_b - fwd_a) / h^2
// (kappa without dt^2: kap / dt2).
cudaError_t image_density_launch(int ny, int nx, int pitch, float idx2, float idy2, int n_shots, const float* adj,
                                 const float* fwd, const float* kap, const float* bx, const float* by, double scale,
                                 double dt2, double* gk, double* gbx, double* gby, cudaStream_t st);
cudaError_t density_chain_launch(int ny, int nx, int pitch, const double* m, const double* rho,
                                 const double* gk, const double* gbx, const double* gby, const uint8_t* mask,
                                 double* g_m, double* g_rho, cudaStream_t st);
// One step of a PML grid (fdtd_step_pml): tables, dt / 2, dt^2 and the face fields.
cudaError_t step_pml_launch(const StepArgs& a, const float* pml, const float* psx,
                            const float* psy, float* psx_next, float* psy_next, cudaStream_t st);
// The PML tables of a padded medium, and coef scaled by q = 1 / (1 + a).
cudaError_t prepare_pml_launch(const double* c, int ny, int nx, int pitch, double dt, double dx, double dy,
                               int cells, double reflection, float* coef, float* pml, cudaStream_t st);
cudaError_t gather_launch(int ny, int pitch, int n_shots, const float* fields, int n_rx,
                          const int32_t* rx_rc, const float* rx_w, float* out,
                          long long shot_stride, long long rx_stride, cudaStream_t st);
cudaError_t scatter_launch(int ny, int pitch, int n_shots, int n_nodes, const int32_t* nodes,
                           const float* w, const float* res, long long shot_stride,
                           long long rx_stride, float* dense, cudaStream_t st);
// g[i] += scale graw[i] / coef[i] (nothing where coef is 0), float64, n elements.
cudaError_t grad_divide_launch(const double* graw, const float* coef, double scale, double* g, long long n,
                               cudaStream_t st);
cudaError_t image_launch(int ny, int nx, int pitch, float idx2, float idy2, float cdiag,
                         int n_shots, const float* adj, const float* fwd, double scale,
                         const float* coef_div, double* g, cudaStream_t st);
cudaError_t prepare_medium_launch(const double* c, int ny, int nx, int pitch, double dt,
                                  double dx, double dy, float* coef, float* mur,
                                  cudaStream_t st);
cudaError_t residual_launch(int n_shots, int n_rx, int n_steps, const float* traces,
                            const float* observed, long long obs_shot_stride,
                            const int32_t* mute, float* residual, double* misfit,
                            cudaStream_t st);
cudaError_t chain_rule_launch(long long n, const double* g, const double* m,
                              const uint8_t* mask, double* out, cudaStream_t st);
// 16-bit checkpoint storage with one power-of-two scale per (field, shot). A slot
// holds src, or src - minus when `minus` is set; dequantisation writes the value,
// or base - value when `base` is set. The engine stores a checkpoint (u_old, u)
// as u and u - u_old: the leapfrog step then keeps its own 11-bit (float16) or
// 8-bit (bfloat16) relative precision instead of inheriting the rounding error
// of two nearly equal fields, which cut the gradient error of 16-bit checkpoints
// about ninefold in a float64 emulation.
cudaError_t quantize_launch(const float* src, const float* minus, void* dst, float* scales, int n_shots,
                            long long per_shot, int store, cudaStream_t st);
cudaError_t dequantize_launch(const void* src, const float* scales, const float* base, float* dst, int n_shots,
                              long long per_shot, int store, cudaStream_t st);

}  // namespace fdtd
