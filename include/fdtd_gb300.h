/*
 * fdtd_gb300.h -- C ABI of the GB300 (sm_103a) engine for the 2-D ring-array
 * wave simulation and its adjoint-state FWI gradient.
 *
 * The reference (scjoshi/SoundWaveSimulation) is pure Python: its engine is
 * fdtd2d/torch_backend.py and its gradient driver is TorchLeastSquaresFWI in
 * invert_ring.py. It has no FFI of its own, so every entry point below names the
 * reference function whose device work it replaces; the Python package
 * soundwavesimulation_gb300 binds these symbols with ctypes and keeps the
 * reference's class and method names on top of them.
 *
 * Conventions
 *  - All functions return 0 (FDTD_OK) or an error code; fdtd_last_error() gives a
 *    readable message for the calling thread.
 *  - Fields are float32, shot-major (shots, ny, pitch) with row = y, column = x.
 *    `pitch` is the row stride in elements: a multiple of 4 and >= nx. Columns
 *    nx..pitch-1 are padding and must hold zeros.
 *  - Traces and residuals are float32 (shots, receivers, steps), as the
 *    reference returns them (fdtd2d/torch_backend.py:769).
 *  - Pointers marked "device" are CUDA device pointers; "host" pointers are read
 *    during the call only. `stream` is a cudaStream_t (NULL = legacy stream).
 *  - No entry point allocates device memory: every device buffer, including the
 *    engine workspace, is owned by the caller.
 */
#ifndef FDTD_GB300_H
#define FDTD_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FDTD_ABI_VERSION 7

enum {
  FDTD_OK = 0,
  FDTD_ERR_INVALID = 1,     /* bad argument (shape, range, CFL, ...) */
  FDTD_ERR_CUDA = 2,        /* a CUDA runtime call failed */
  FDTD_ERR_WORKSPACE = 3,   /* workspace missing or too small */
  FDTD_ERR_UNSUPPORTED = 4, /* configuration outside what the kernels support */
  FDTD_ERR_STATE = 5        /* call order violated (e.g. adjoint before forward) */
};

enum { FDTD_STORE_F32 = 0, FDTD_STORE_F16 = 1, FDTD_STORE_BF16 = 2 };

/* Grid and medium. `coef` and `mur` come from fdtd_prepare_medium, or for a grid
   with a PML layer from fdtd_prepare_medium_pml. */
typedef struct fdtd_grid {
  int32_t ny, nx, pitch;
  double dx, dy, dt;
  const float* coef; /* device (ny, pitch): b = (c * dt / dy)^2, the update coefficient of the
                        stencil in units of 1/dy^2 (Q = dy^2 lap, see fdtd_step); with a PML
                        q b, q = 1 / (1 + a), a = dt (sigma_x + sigma_y) / 2 */
  const float* mur;  /* device, 2 * (2 ny + 2 nx + 8) floats: k_left[ny], k_right[ny],
                        k_bottom[nx], k_top[nx], corner_kx[4], corner_ky[4] (corners
                        in the order (0,0), (0,nx-1), (ny-1,0), (ny-1,nx-1)), then in
                        the same layout the ratios coef_edge / coef_inner used by the
                        adjoint in w = coef * l form */
  const float* pml;  /* NULL (Mur edges, the reference's boundary), or device PML tables of
                        4 (nx + ny) floats: per column dt sigma_x / 2 at the cell centre and
                        at the left face, the face decay (1 - sigma dt / 2) / (1 + sigma dt / 2)
                        and the forcing scale 2 dy^2 / (dx^2 (1 + sigma dt / 2)); then per row
                        the same for y (forcing scale 2 / (1 + sigma dt / 2)). The grid then has no Mur edges: it ends in a rigid wall
                        behind the layer. */
  int32_t pml_cells; /* layer thickness in cells on every side (with pml) */
} fdtd_grid;

/* Bilinear receivers (host arrays of length n). Receiver i samples rows
   row0[i], row0[i]+1 and columns col0[i], col0[i]+1 with weights
   w[4i..4i+3] = (w00, w10, w01, w11) as in RingArray._init_bilinear
   (fdtd2d/array.py:60-76). */
typedef struct fdtd_receivers {
  int32_t n;
  const int32_t* row0;
  const int32_t* col0;
  const float* w;
} fdtd_receivers;

/* Soft sources: `per_shot` injection entries per shot (host arrays of shape
   (n_shots, per_shot)); entry j of shot s adds w * waveforms[wave, step] to node
   (row, col) before the Mur edges are applied. wave = -1 marks an unused entry.
   Nearest-node injection (fdtd2d/torch_backend.py:517) is one entry of weight 1;
   the bilinear source (desmond/src/phase2_numerics.py:107-118) is four. */
typedef struct fdtd_sources {
  int32_t per_shot;
  const int32_t* row;
  const int32_t* col;
  const float* w;
  const int32_t* wave;
  const float* waveforms; /* device (n_waves, waveform_len) */
  int32_t n_waves;
  int32_t waveform_len;   /* samples per waveform; steps beyond it inject 0 */
} fdtd_sources;

typedef struct fdtd_problem {
  fdtd_grid grid;
  int32_t n_shots;
  int32_t n_steps;
  fdtd_receivers rx;
  fdtd_sources src;
} fdtd_problem;

/* Launch shape of the temporally blocked engine. Zero fields take defaults. */
typedef struct fdtd_tuning {
  int32_t rows_per_lane;    /* rows each lane keeps in registers: 4 or 8 */
  int32_t warps;            /* warps per CTA, 2..16 (2..32 with 4 rows per lane); region height = warps * rows_per_lane */
  int32_t steps_per_launch; /* leapfrog steps per HBM round trip (temporal block) */
  int32_t ckpt_every;       /* checkpoint spacing in steps, rounded up to a multiple of
                               steps_per_launch; 0 = about sqrt(2 nt) */
  int32_t ckpt_store;       /* FDTD_STORE_F32 / _F16 / _BF16; 16-bit checkpoints hold u and the
                               step u - u_old, each with a power-of-two scale per shot */
  int32_t ctas_per_sm;      /* persistent grid = SMs * ctas_per_sm; 0 = 1 */
  int32_t eager;            /* 0 (default): fdtd_forward / fdtd_adjoint capture their launch
                               sequence once per set of output pointers and replay it as a
                               CUDA graph; 1: launch every kernel from the host */
  int32_t step_sync;        /* FDTD_SYNC_*: how the warps of a CTA meet after every step */
  int32_t kept_segments;    /* gradient plans of grids without PML: the last kept_segments
                               checkpoint segments of the pass have their stencil stream
                               written by the forward with checkpoints and kept, so the
                               adjoint recomputes only the segments before them; each takes
                               ckpt_every * n_shots * ny * pitch * 4 bytes of workspace.
                               0 = 1 (the recompute's own buffer), negative = none;
                               fdtd_plan_tuning reports the count in effect (-1: none) */
} fdtd_tuning;

/* Step synchronisation of the temporally blocked kernel. After every leapfrog step
   a warp has published the first and last row of its band, which only the warps
   above and below read: FDTD_SYNC_PAIR meets each neighbouring pair of warps on
   its own hardware barrier, so warps further apart drift by up to their distance
   in steps; FDTD_SYNC_CTA meets the whole CTA. FDTD_SYNC_AUTO takes PAIR up to
   16 warps (15 named barriers) and CTA beyond. */
#define FDTD_SYNC_AUTO 0
#define FDTD_SYNC_CTA 1
#define FDTD_SYNC_PAIR 2

typedef struct fdtd_plan fdtd_plan; /* opaque host-side execution plan */

/* Variable density (no reference counterpart in 2-D: the reference propagates
   with constant density; its 1-D solver, 1DWaveSimulation.py:116-143, gives the
   conservative form u_tt = rho c^2 div((1/rho) grad u) with 1/rho on the faces as
   2 / (rho_a + rho_b)). fdtd_prepare_density fills the three device arrays; an
   outer face takes its edge cell's rho. At constant rho the operator is the
   reference's stencil. */
typedef struct fdtd_density {
  const float* kappa; /* device (ny, pitch): rho c^2 dt^2 */
  const float* bx;    /* device (ny, pitch + 4): 1/rho on the face between columns x-1 and x, x = 0..nx */
  const float* by;    /* device (ny + 1, pitch): 1/rho on the face between rows y-1 and y, y = 0..ny */
} fdtd_density;

/* ---------------------------------------------------------------- basics */
int32_t fdtd_abi_version(void);
const char* fdtd_last_error(void);

/* Sound speed (device float64 (ny, nx), row stride nx) -> coef and Mur
   coefficients, computed in float64 and rounded to float32.
   Replaces TorchScalarWave2D.set_c (fdtd2d/torch_backend.py:158-168) and
   TorchFDTD2D._refresh_boundaries (fdtd2d/torch_backend.py:264-275). */
int32_t fdtd_prepare_medium(const double* c, int32_t ny, int32_t nx, int32_t pitch,
                            double dt, double dx, double dy,
                            float* coef, float* mur, void* stream);

/* The same for a grid padded by a PML layer of `cells` cells on every side (no
   reference counterpart: the reference has first-order Mur edges only). c is the
   padded medium; the damping grows as sigma_max (depth / cells)^2 with
   sigma_max = 3 max(c) ln(1 / reflection) / (2 cells h) per axis. Writes coef =
   q (c dt / dy)^2, the Mur table (unused by PML grids) and the PML tables
   (device, 4 (nx + ny) floats) that fdtd_grid.pml points to. */
int32_t fdtd_prepare_medium_pml(const double* c, int32_t ny, int32_t nx, int32_t pitch,
                                double dt, double dx, double dy, int32_t cells, double reflection,
                                float* coef, float* mur, float* pml, void* stream);

/* kappa, the face coefficients and the Mur table (from c, as fdtd_prepare_medium)
   of a medium with sound speed c and density rho (device float64 (ny, nx)). */
int32_t fdtd_prepare_density(const double* c, const double* rho, int32_t ny, int32_t nx, int32_t pitch,
                             double dt, double dx, double dy, float* kappa, float* bx, float* by,
                             float* mur, void* stream);

/* ------------------------------------------------- one-step (plain) kernels */

/* One leapfrog step for n_shots shots, Mur edges included. With the stencil in
   units of 1/dy^2, Q(u) = (u_d + u_u) + ratio (u_l + u_r) - 2 (1 + ratio) u,
   ratio = dy^2 / dx^2 (Q = dy^2 lap(u), zero beyond the grid), and coef = b =
   (c dt / dy)^2:
     forward: u_next = 2u - u_old + coef * Q(u) + sources  (= (c dt)^2 lap(u))
     adjoint = 1: u_next = 2u - u_old + Q(coef * u) + sources
     adjoint = 2: the same adjoint carried as w = coef * u:
                  w_next = 2w - w_old + coef * Q(w) + coef * sources, with the
                  Mur edges rescaled by the coef ratios (the fused engine's form)
   Sources: `src_*` are device arrays of shape (n_shots, src_per_shot) (row, col,
   weight, waveform index) and inject w * waveforms[wave * waveform_len + step];
   `dense` (device (n_shots, ny, pitch), nullable) is added as a field.
   u_next must not alias u_old or u.
   Replaces _advance_field (fdtd2d/torch_backend.py:177-233),
   _advance_field_batch (493-522) and _advance_adjoint_field_batch (525-537). */
int32_t fdtd_step(const fdtd_grid* grid, int32_t n_shots,
                  const float* u_old, const float* u, float* u_next,
                  int32_t src_per_shot, const int32_t* src_row, const int32_t* src_col,
                  const float* src_w, const int32_t* src_wave,
                  const float* waveforms, int32_t waveform_len, int32_t step,
                  const float* dense, int32_t adjoint, void* stream);

/* One leapfrog step of a PML grid (grid->pml set): the face fields psi_x, psi_y
   (device (n_shots, ny, pitch), zero at the start) step from psx / psy into
   psx_next / psy_next together with the field; no Mur edges. Sources and
   `adjoint` (0 forward, 2 the w = coef * l adjoint) as fdtd_step. The fused
   engine computes the same values bit for bit. No reference counterpart. */
int32_t fdtd_step_pml(const fdtd_grid* grid, int32_t n_shots,
                      const float* u_old, const float* u, float* u_next,
                      const float* psx, const float* psy, float* psx_next, float* psy_next,
                      int32_t src_per_shot, const int32_t* src_row, const int32_t* src_col,
                      const float* src_w, const int32_t* src_wave,
                      const float* waveforms, int32_t waveform_len, int32_t step,
                      const float* dense, int32_t adjoint, void* stream);

/* fdtd_step with variable density: u_next = 2u - u_old + kappa D(b, u) + sources,
   the reference's Mur edges (local sound speed); adjoint = 1 gives the reference's
   adjoint form l_next = 2l - l_old + D(b, kappa l) + sources (adjoint = 2 is not
   offered). No reference counterpart in 2-D. */
int32_t fdtd_step_density(const fdtd_grid* grid, const fdtd_density* density, int32_t n_shots,
                          const float* u_old, const float* u, float* u_next,
                          int32_t src_per_shot, const int32_t* src_row, const int32_t* src_col,
                          const float* src_w, const int32_t* src_wave,
                          const float* waveforms, int32_t waveform_len, int32_t step,
                          const float* dense, int32_t adjoint, void* stream);

/* Bilinear receiver samples of a field batch:
   out[s * out_shot_stride + r * out_rx_stride] for s < n_shots, r < n_rx.
   rx_rc is device int32 (n_rx, 2) = (row0, col0), rx_w device float (n_rx, 4).
   Replaces _gather_receivers (fdtd2d/torch_backend.py:540-548) and
   TorchRingSampler.record / record_batch (368-387). */
int32_t fdtd_gather(const fdtd_grid* grid, int32_t n_shots, const float* fields,
                    int32_t n_rx, const int32_t* rx_rc, const float* rx_w,
                    float* out, int64_t out_shot_stride, int64_t out_rx_stride,
                    void* stream);

/* Transpose of fdtd_gather: writes, for every node in the receiver tap table,
   dense[s, node] = sum of w * residual[s * res_shot_stride + rx * res_rx_stride]
   over the taps that land on the node (a fixed order, so the result is
   deterministic). Nodes outside the table are left untouched: zero `dense`
   once, then reuse it. tap_nodes is device int32 (n_nodes, 10) =
   (row, col, rx_0, ..., rx_7) with -1 for unused receivers, tap_w device
   float (n_nodes, 8). fdtd_tap_table builds both.
   Replaces the scatter of _adjoint_inject_batch (fdtd2d/torch_backend.py:563-577)
   and TorchRingSampler.record_adjoint_batch (389-418). */
int32_t fdtd_scatter(const fdtd_grid* grid, int32_t n_shots, int32_t n_nodes,
                     const int32_t* tap_nodes, const float* tap_w,
                     const float* residual, int64_t res_shot_stride, int64_t res_rx_stride,
                     float* dense, void* stream);

/* Imaging condition g[y, x] += scale * sum_s adj[s, y, x] * lap(fwd[s])[y, x]
   with the zero-padded Laplacian at every node; g is float64 (ny, pitch).
   Replaces the imaging term of _adjoint_image_batch (fdtd2d/torch_backend.py:
   583-598). */
int32_t fdtd_image(const fdtd_grid* grid, int32_t n_shots, const float* adj,
                   const float* fwd, double scale, double* g, void* stream);

/* Host helper: builds the deterministic receiver tap table used by
   fdtd_scatter and the fused engine (unique nodes, up to 8 receivers each).
   On input *n_nodes is the capacity of the output arrays (4 * n_rx suffices). */
int32_t fdtd_tap_table(int32_t ny, int32_t nx, const fdtd_receivers* rx,
                       int32_t* tap_nodes, float* tap_w, int32_t* n_nodes);

/* ------------------------------------------------------- fused engine */

/* Builds the host-side plan: tiling, tap and source tables, checkpoint
   schedule and workspace layout. for_gradient = 1 reserves checkpoints,
   the recompute segment buffer and the adjoint state. */
int32_t fdtd_plan_create(const fdtd_problem* problem, const fdtd_tuning* tuning,
                         int32_t for_gradient, fdtd_plan** plan);
int32_t fdtd_plan_destroy(fdtd_plan* plan);
int32_t fdtd_plan_workspace_bytes(const fdtd_plan* plan, size_t* bytes);
/* Reports the resolved tuning (defaults filled in) and the checkpoint spacing. */
int32_t fdtd_plan_tuning(const fdtd_plan* plan, fdtd_tuning* tuning);
/* Binds a caller-owned device workspace (256-byte aligned) and uploads the
   tables into it; synchronises `stream` once. */
int32_t fdtd_plan_bind(fdtd_plan* plan, void* workspace, size_t bytes, void* stream);
/* Updates the medium and source waveform pointers of a bound plan (same shapes);
   checkpoints become stale. The plan's captured CUDA graphs read the medium
   through these pointers and are kept while the pointers stay the same (values
   updated in place); a changed pointer makes the next pass capture again. */
int32_t fdtd_plan_set_medium(fdtd_plan* plan, const float* coef, const float* mur,
                             const float* waveforms);

/* Batched forward of every shot over n_steps with the fused temporally blocked
   kernel. traces: (n_shots, n_rx, n_steps), device memory or pinned host memory
   (which the kernels then write directly). u_prev_out / u_out (nullable, device
   (n_shots, ny, pitch)) receive the last two fields. save_checkpoints = 1 keeps
   what a later fdtd_adjoint needs: the checkpoints of the segments it will
   recompute and the stencil stream of the kept segments (kept_segments).
   Replaces simulate_shots_batch (fdtd2d/torch_backend.py:736-770) and
   forward_store_batch (invert_ring.py:422-455). */
int32_t fdtd_forward(fdtd_plan* plan, float* traces, float* u_prev_out, float* u_out,
                     int32_t save_checkpoints, void* stream);

/* Reverse-time adjoint of the last checkpointed forward: injects `residual`
   (device (n_shots, n_rx, n_steps)), recomputes each checkpoint segment that the
   forward did not keep and adds dt^2 * sum_{shots, n >= 1} adj^n * lap(u^{n-1})
   into grad_c2 (device float64 (ny, pitch)).
   Replaces _adjoint_accumulate_batch (invert_ring.py:683-701) with
   store_every = 1. */
int32_t fdtd_adjoint(fdtd_plan* plan, const float* residual, double* grad_c2, void* stream);

/* residual = traces - observed with channel mute[s] zeroed (mute[s] < 0: none),
   misfit[0] += 0.5 * sum(residual^2) in float64. Arrays (n_shots, n_rx, n_steps);
   residual may alias traces. observed_shot_stride lets `observed` be a row
   subset of a larger gather. mute is device int32 (n_shots).
   Replaces TorchLeastSquaresFWI._residual_batch and the misfit sum
   (invert_ring.py:603-609, 651). */
int32_t fdtd_residual_misfit(int32_t n_shots, int32_t n_rx, int32_t n_steps,
                             const float* traces, const float* observed,
                             int64_t observed_shot_stride, const int32_t* mute,
                             float* residual, double* misfit, void* stream);

/* g_m = -grad_c2 / m^2 where mask != 0, else 0 (float64, n elements, all device;
   mask may be NULL). Replaces invert_ring.py:657-659 without regularisation. */
int32_t fdtd_chain_rule(int64_t n, const double* grad_c2, const double* m,
                        const uint8_t* mask, double* g_m, void* stream);

/* ------------------------------------------------- plain per-shot engine */

/* The plain form: each shot separately, one launch per step per kernel
   (step, then gather), traces as fdtd_forward. Workspace: 3 fields of one shot.
   Replaces simulate_shot (fdtd2d/torch_backend.py:443-474) looped over shots. */
int32_t fdtd_forward_plain(const fdtd_problem* problem, float* traces,
                           void* workspace, size_t bytes, void* stream);
size_t fdtd_forward_plain_workspace(const fdtd_problem* problem);

/* The plain per-shot gradient: for each shot a forward that keeps every field
   (one step + one gather launch per step), the residual against `observed`
   (device (n_shots, n_rx, n_steps)) with channel mute[s] zeroed, then one
   scatter + adjoint step + imaging launch per step; adds the misfit into
   misfit[0] and dt^2 sum adj^n lap(u^{n-1}) into grad_c2 (float64 (ny, pitch)).
   The structure of TorchLeastSquaresFWI._adjoint_accumulate with full float32
   history (invert_ring.py:668-681), on the one-step kernels. */
int32_t fdtd_gradient_plain(const fdtd_problem* problem, const float* observed,
                            const int32_t* mute, double* misfit, double* grad_c2,
                            void* workspace, size_t bytes, void* stream);
size_t fdtd_gradient_plain_workspace(const fdtd_problem* problem);

/* The plain per-shot forms with variable density (workspaces as fdtd_forward_plain
   / fdtd_gradient_plain). The gradient adds dt^2 sum adj^n D(b, u^{n-1}) into
   g_kappa (float64 (ny, pitch)) and, per face, dt^2 sum (adj_a kappa_a - adj_b
   kappa_b) (u_b - u_a) / h^2 into g_bx (float64 (ny, pitch + 4)) and g_by (float64
   (ny + 1, pitch)), kappa without dt^2 here: the derivatives of the misfit with
   respect to rho c^2 and to the face coefficients 1/rho, the pairing of adjoint
   and forward fields of the reference's imaging (invert_ring.py:683-701). No
   reference counterpart in 2-D. */
int32_t fdtd_forward_plain_density(const fdtd_problem* problem, const fdtd_density* density, float* traces,
                                   void* workspace, size_t bytes, void* stream);
int32_t fdtd_gradient_plain_density(const fdtd_problem* problem, const fdtd_density* density,
                                    const float* observed, const int32_t* mute, double* misfit,
                                    double* g_kappa, double* g_bx, double* g_by,
                                    void* workspace, size_t bytes, void* stream);

/* g_m = -g_kappa rho / m^2 and g_rho = g_kappa / m - sum over the cell's faces of
   g_b b^2 / 2 (b^2 on an outer face), zero where mask == 0 (nullable): the chain
   rule to slowness squared m = 1 / c^2 and density rho (float64, m and rho
   (ny, nx), the gradients in the layouts above). */
int32_t fdtd_density_chain_rule(int32_t ny, int32_t nx, int32_t pitch, const double* m, const double* rho,
                                const double* g_kappa, const double* g_bx, const double* g_by,
                                const uint8_t* mask, double* g_m, double* g_rho, void* stream);

/* Size of the fixed device scratch behind fdtd_forward_plain_static: three
   fields of one shot plus the receiver and source tables must fit (about
   1180 x 1180 cells at most; 1024 x 1024 with 512 receivers uses ~12 MiB). */
#define FDTD_STATIC_SCRATCH_BYTES (16u << 20)

/* fdtd_forward_plain for callers that cannot allocate device memory (no
   counterpart in the reference). Same problem and traces as
   fdtd_forward_plain, no workspace: the scratch is a file-scope device array of
   FDTD_STATIC_SCRATCH_BYTES that every GPU loading the library holds until exit.
   Calls no cudaMalloc, cudaFree or allocating library routine. Problems that do
   not fit return FDTD_ERR_WORKSPACE with a message; bad receivers, source
   nodes or waveform indices return FDTD_ERR_INVALID before any device work. The
   first call on a device looks up the array's address (cudaGetSymbolAddress,
   that device current) and caches it: make that first call before any stream
   capture. The cached address belongs to the device's primary context; a
   cudaDeviceReset or a non-primary context is not supported. Every call copies
   the receiver and source tables from the host arrays into the array and
   synchronises `stream` before the time loop. All calls share the array and it
   keeps the last call's contents (each shot clears the fields it uses); calls
   that overlap on the GPU race on it. */
int32_t fdtd_forward_plain_static(const fdtd_problem* problem, float* traces, void* stream);

/* ------------------------------------------------------- launch-shape search */

/* Device bytes fdtd_autotune needs for this problem: the largest probe plan's
   workspace plus its traces and a gradient buffer. */
size_t fdtd_autotune_workspace_bytes(const fdtd_problem* problem, int32_t for_gradient, int32_t launches);

/* Times every candidate launch shape (rows per lane 8 x 16 / 12 / 10 warps and
   4 x 32 / 16 warps, steps per launch 6 .. 23) that the planner accepts for this
   grid on `launches` temporal blocks of the problem (a forward; with
   for_gradient a forward with checkpoints plus the adjoint), each after one
   untimed pass, averaged over `repeats` passes with CUDA events on `stream`, and
   writes the fastest into *best (its rate in Gcell-updates/s into *best_rate,
   nullable). Optional report: on input *n_tried is the capacity of tried /
   rates (nullable), on output the number written. The workspace (device, 256-
   byte aligned, fdtd_autotune_workspace_bytes) is reused by every probe; the
   call allocates no device memory and synchronises `stream`.
   The reference has no tuner: its batch size comes from auto_batch_size
   (fdtd2d/torch_backend.py:773-789) and its step from torch.compile
   (fdtd2d/torch_backend.py:257-262). */
int32_t fdtd_autotune(const fdtd_problem* problem, int32_t for_gradient, int32_t launches, int32_t repeats,
                      void* workspace, size_t bytes, fdtd_tuning* best, double* best_rate,
                      fdtd_tuning* tried, double* rates, int32_t* n_tried, void* stream);

/* ------------------------------------------------------- tiling (host) */

/* The 1-D tiler of the fused engine, exposed for tests: covers [0, n) with
   regions of `region` cells whose origins are multiples of `align`, owned
   ranges that partition [0, n) and lie at least `halo` cells inside interior
   region borders, and keeps every domain edge row together with its inner
   neighbour inside one band of `band` cells. out holds 4 ints per tile:
   (region origin, owned begin, owned end, flags). */
int32_t fdtd_tile_axis(int32_t n, int32_t region, int32_t align, int32_t halo,
                       int32_t band, int32_t max_tiles, int32_t* out, int32_t* n_tiles);

/* Uneven batches: several bound plans (grids of different sizes, step counts and
   steps per launch, but one rows_per_lane / warps shape) advanced together; each
   round merges the next temporally blocked launch of every plan into one launch
   per kernel mode, so small grids share the GPU instead of running one after
   another. traces / residuals / grads hold one pointer per plan (as for
   fdtd_forward / fdtd_adjoint); the device workspace (size from
   fdtd_group_workspace_bytes) holds the launches' parameter tables. Engine-
   specific: the reference runs the stages of its multiscale driver in turn
   (invert_ring.py:1037-1045). */
size_t fdtd_group_workspace_bytes(fdtd_plan* const* plans, int32_t n);
int32_t fdtd_group_forward(fdtd_plan* const* plans, int32_t n, float* const* traces, int32_t save_checkpoints,
                           void* workspace, size_t bytes, void* stream);
int32_t fdtd_group_adjoint(fdtd_plan* const* plans, int32_t n, const float* const* residuals,
                           double* const* grads, void* workspace, size_t bytes, void* stream);

/* ------------------------------------------------- inversion helpers */

/* Adds the Tikhonov (1/2 alpha ||grad m||^2) and smoothed total-variation
   (tv sum(sqrt(|grad m|^2 + tv_eps^2) - tv_eps)) gradients of the slowness squared
   m (float64 (ny, nx), device) into `grad` on the mask (uint8, non-zero = inside)
   and sets grad to 0 outside it; adds both values into the device double `value`.
   Replaces tikhonov / total_variation (fdtd2d/inversion/misfit.py:19-71) and the
   host gradient assembly of misfit_and_grad (invert_ring.py:655-659). */
int32_t fdtd_regularization(int32_t ny, int32_t nx, const double* m, const uint8_t* mask, double alpha,
                            double tv, double tv_eps, double* grad, double* value, void* stream);
/* m = clip(m, m_min, m_max) inside the mask, m_exterior outside
   (TorchLeastSquaresFWI.project, invert_ring.py:559-565). */
int32_t fdtd_project(int64_t n, double* m, const uint8_t* mask, double m_min, double m_max,
                     double m_exterior, void* stream);
/* One projected Adam step on the mask (invert_ring.py:842-853), iteration >= 1;
   first / second are the moment arrays (zero before the first step). */
int32_t fdtd_adam_step(int64_t n, double* m, const double* grad, const uint8_t* mask, double* first,
                       double* second, double learning_rate, double beta1, double beta2, double epsilon,
                       int32_t iteration, double m_min, double m_max, double m_exterior, void* stream);
/* Bicubic transfer of m (float64, device) between grid levels in physical
   coordinates: src_x / src_y and dst_x / dst_y are the device cell-centre axes;
   target points outside the source grid get `background`. Replaces
   resize_slowness (invert_ring.py:1048-1068), which calls torch grid_sample
   (bicubic, border padding, align_corners). */
int32_t fdtd_resize_slowness(const double* src, int32_t src_ny, int32_t src_nx, const double* src_x,
                             const double* src_y, double* dst, int32_t dst_ny, int32_t dst_nx,
                             const double* dst_x, const double* dst_y, double background, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* FDTD_GB300_H */
