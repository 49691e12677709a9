// Device-side arithmetic and parameter blocks shared by every kernel of the
// engine.
//
// All float32 arithmetic of the update is written with explicit round-to-nearest
// intrinsics (no compiler contraction choices), so the one-step kernels, the
// temporally blocked kernel and the checkpoint recompute produce bit-identical
// fields, traces and Laplacians for the same inputs.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace fdtd {

// ---------------------------------------------------------------- arithmetic

// The update stencil in units of 1/dy^2 (the conv2d kernel of
// fdtd2d/torch_backend.py:124-132 with zero padding, times dy^2):
//   Q(u) = (d + u) + ratio (l + r) + qdiag c,  ratio = dy^2 / dx^2,
//   qdiag = -2 (1 + ratio),  lap(u) = Q(u) / dy^2.
// The coefficient array holds b = (c dt / dy)^2, rounded once from float64, so the
// leapfrog u+ = 2u - u- + b Q(u) needs no per-step multiply by 1/dy^2: six float32
// operations per cell, and one rounding fewer per step than b' lap(u) with
// b' = (c dt)^2. With dx = dy, ratio = 1 and qdiag = -4 are exact.
__device__ __forceinline__ float nbrq(float l, float r, float d, float u, float ratio) {
  return __fmaf_rn(__fadd_rn(l, r), ratio, __fadd_rn(d, u));
}

__device__ __forceinline__ float lapq(float c, float l, float r, float d, float u, float ratio, float qdiag) {
  return __fmaf_rn(c, qdiag, nbrq(l, r, d, u, ratio));
}

// Off-centre part of the 5-point Laplacian, (l + r) / dx^2 + (d + u) / dy^2.
__device__ __forceinline__ float nbr4(float l, float r, float d, float u, float idx2, float idy2) {
  return __fmaf_rn(__fadd_rn(d, u), idy2, __fmul_rn(__fadd_rn(l, r), idx2));
}

// Full 5-point Laplacian nbr4 - 2 (1/dx^2 + 1/dy^2) c: the conv2d kernel of
// fdtd2d/torch_backend.py:124-132 with zero padding.
__device__ __forceinline__ float lap5(float c, float l, float r, float d, float u,
                                      float idx2, float idy2, float cdiag) {
  return __fmaf_rn(c, cdiag, nbr4(l, r, d, u, idx2, idy2));
}

// Forward leapfrog u+ = 2u - u_old + (c dt)^2 lap(u) (fdtd2d/torch_backend.py:516),
// as 2u - u_old + b Q(u) (coef = b, lap = Q above). 2u - u_old is formed with one
// rounding (2u is exact). The factor 2 must stay exact: folding it into a
// per-cell 2 + b qdiag rounded to float32 shifts every mode's frequency by a
// fixed relative amount, which accumulates coherently over thousands of steps.
__device__ __forceinline__ float leap(float c, float p, float coef, float lap) {
  return __fmaf_rn(coef, lap, __fmaf_rn(2.0f, c, -p));
}

// Adjoint leapfrog 2l - l_old + lap((c dt)^2 l)  (fdtd2d/torch_backend.py:531-532),
// as 2l - l_old + Q(b l); the coefficient is already inside the operand.
__device__ __forceinline__ float leap_adj(float c, float p, float lap) {
  return __fadd_rn(__fsub_rn(__fadd_rn(c, c), p), lap);
}

// First-order Mur edge u_in + k (un_in - u_edge)  (fdtd2d/torch_backend.py:482-489).
__device__ __forceinline__ float mur(float u_in, float k, float un_in, float u_edge) {
  return __fmaf_rn(k, __fsub_rn(un_in, u_edge), u_in);
}

// The same Mur update for the adjoint carried as w = coef l: with
// r = coef_edge / coef_inner, coef_edge * (l_in + k (l_in' - l_edge)) equals
// r w_in + k (r w_in' - w_edge).
__device__ __forceinline__ float murw(float r, float w_in, float k, float wn_in, float w_edge) {
  return mur(__fmul_rn(r, w_in), k, __fmul_rn(r, wn_in), w_edge);
}

__device__ __forceinline__ float corner_avg(float fx, float fy) {
  return __fmul_rn(0.5f, __fadd_rn(fx, fy));
}

// Bilinear receiver sample (fdtd2d/torch_backend.py:543-548).
__device__ __forceinline__ float gather4(float a, float b, float c, float d,
                                        float w00, float w10, float w01, float w11) {
  return __fmaf_rn(d, w11, __fmaf_rn(c, w01, __fmaf_rn(b, w10, __fmul_rn(a, w00))));
}

// Accumulates one weighted injection term.
__device__ __forceinline__ float inj_acc(float acc, float w, float v) {
  return __fmaf_rn(w, v, acc);
}

__device__ __forceinline__ float inj_add(float un, float inj) { return __fadd_rn(un, inj); }

// ---------------------------------------------------------------- PML
//
// The second-order PML of a grid padded by a damping layer (no reference
// counterpart; the reference has first-order Mur edges only): stretched
// coordinates s = 1 + sigma / (i omega) per axis, multiplied through by s_x s_y,
//   u_tt + (sx + sy) u_t + sx sy u = c^2 (lap u + d/dx phi_x + d/dy phi_y),
//   phi_x_t = -sx phi_x + (sy - sx) du/dx,  phi_y_t = -sy phi_y + (sx - sy) du/dy,
// with phi on the cell faces at half steps, stored as psi = phi / h: psi_x of cell
// (y, x) lives on its left face, psi_y on its bottom face. Tables per column
// (sigma_x at the centre and the left face, the face decay and forcing scale, the
// latter times dy^2) and per row (the same for y) come from fdtd_prepare_medium_pml; the update factors
// of a cell follow from sigma_x, sigma_y at its centre. Where sigma = 0 every
// factor is exactly 1 or 2 and psi stays 0, so the update is bit for bit the
// plain leapfrog (leap above).

// One face value psi+ = alpha psi + (sigma_other - sigma_face) beta du, with the
// sigmas scaled by dt / 2 and beta by 2 / dt in the tables.
__device__ __forceinline__ float pml_face(float alpha, float psi, float sig_other, float sig_face, float beta,
                                          float du) {
  return __fmaf_rn(alpha, psi, __fmul_rn(__fmul_rn(__fsub_rn(sig_other, sig_face), beta), du));
}

// Factors A = q (2 - dt^2 sx sy) = q (2 - 4 hx hy) and M = (1 - a) q, with
// a = hx + hy and q = 1 / (1 + a), of the cell update u+ = K (Q + div) + A u - M u-;
// the tables hold hx = dt sigma_x / 2 and hy = dt sigma_y / 2 at the cell centre,
// the coefficient table K = q (c dt / dy)^2 (from float64), and the face fields carry
// the factor dy^2 of Q (their forcing scale includes it). q takes the hardware's
// approximate reciprocal (the damping factors need no correctly rounded one), and is
// exactly 1 where a = 0, so that there A = 2 and M = 1 exactly.
__device__ __forceinline__ void pml_factors(float hx, float hy, float& A, float& M) {
  const float a = __fadd_rn(hx, hy);
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(__fadd_rn(1.0f, a)));
  const float q = (a == 0.0f) ? 1.0f : r;
  A = __fmul_rn(q, __fmaf_rn(-4.0f, __fmul_rn(hx, hy), 2.0f));
  M = __fmul_rn(__fsub_rn(1.0f, a), q);
}

// div psi = (psi_x right - psi_x left) + (psi_y top - psi_y bottom)
__device__ __forceinline__ float pml_div(float pxl, float pxr, float pyb, float pyt) {
  return __fadd_rn(__fsub_rn(pxr, pxl), __fsub_rn(pyt, pyb));
}

// u+ = K (Q + div) + (A u - M u-): the plain leap when A = 2, M = 1, div = 0.
__device__ __forceinline__ float pml_leap(float c, float p, float K, float A, float M, float lap, float div) {
  return __fmaf_rn(K, __fadd_rn(lap, div), __fmaf_rn(A, c, -__fmul_rn(M, p)));
}

// ------------------------------------------------------------ parameters

constexpr int MODE_FWD = 0;  // forward: sources in, receiver traces out
constexpr int MODE_REC = 1;  // recompute: sources in, Laplacian of every step out
constexpr int MODE_ADJ = 2;  // adjoint: residual in, imaging into the gradient
// forward that also writes the recompute's stencil stream: a gradient plan's forward
// over the segments whose stream it keeps (their recompute is then skipped)
constexpr int MODE_FWDQ = 3;

// Modes that record receiver traces / write the stencil stream.
__host__ __device__ constexpr bool mode_traces(int m) { return m == MODE_FWD || m == MODE_FWDQ; }
__host__ __device__ constexpr bool mode_stream(int m) { return m == MODE_REC || m == MODE_FWDQ; }

constexpr int RX = 128;       // region width: 32 lanes x 4 columns
constexpr int TAP_C = 8;      // receivers sharing one tap node
constexpr int SRC_C = 4;      // source entries sharing one node

// Tile flags. TF_PML: the region holds cells of a PML layer.
constexpr int TF_LEFT = 1, TF_RIGHT = 2, TF_BOTTOM = 4, TF_TOP = 8, TF_OUTSIDE = 16, TF_PML = 32;
constexpr int TF_MUR = TF_LEFT | TF_RIGHT | TF_BOTTOM | TF_TOP;

// PML tables (device, 4 (nx + ny) floats): per column sigma_x at the centre, at
// the left face, the psi_x decay and forcing scale; then the same per row for y.
constexpr int PML_TABLES = 4;

struct TbTile {
  int rx0, ry0;          // region origin (rx0 multiple of 4)
  int ox0, ox1, oy0, oy1;  // owned (written) cells
  int flags;
  int tap_off, ntap;     // receiver tap nodes inside the region
  int rxl_off, nrxl;     // receivers with a tap inside the region
  int rec_off, nrec;     // receivers whose samples this tile records
  int nrow;              // staged tap rows: (thread, band row) pairs holding a tap node
  int pad1, pad2;
};

struct TbTap {           // one receiver tap node inside a tile
  int packed;            // (thread << 8) | (row_in_lane * 4 + column_in_lane)
  int srow;              // staged tap row holding this node (its float is srow * 4 + column)
  int rloc[TAP_C];       // tile-local receiver index of each contribution, -1 = none
  float w[TAP_C];
};

struct TbRec {           // one receiver recorded by a tile
  int rg;                // global receiver index
  int slot[4];           // staged floats (srow * 4 + column) of (r0,c0), (r0,c1), (r1,c0), (r1,c1)
  float w[4];
};

struct SrcNode {         // one injection node of one shot
  int row, col;
  int wave[SRC_C];       // waveform index per entry, -1 = none
  float w[SRC_C];
};

// Per (tile, thread): the band rows holding receiver tap nodes and the first
// staged tap row (0x7fffffff without taps); shot-independent, built by the plan.
struct TbMask {
  unsigned mask;
  int base;
};

struct SrcTap {          // one injection node of one shot inside one tile
  int packed;            // (thread << 8) | (row_in_lane * 4 + column_in_lane)
  int srow;              // staged source row (its float is srow * 4 + column)
  int node;              // index into the shot's node list
  int pad;
};

struct TbParams {
  // grid
  int ny, nx, pitch;
  float idx2, idy2, cdiag;
  float ratio, qdiag;    // the stencil Q in units of 1/dy^2 (see nbrq)
  const float* coef;     // b = (c dt / dy)^2
  const float* mur;
  // tiling
  const TbTile* tiles;
  int ntiles, nshots, nwarps;
  const TbTap* taps;
  const TbMask* tmask;   // (ntiles, nwarps * 32)
  const int* rxl;
  const TbRec* recs;
  int nrow_max, nrxl_max, tmax;  // nrow_max: staged tap rows of the largest tile
  int adj_coef;          // adjoint: 1 = coefficient tile in shared memory, 0 = read through L1
  int pair_sync;         // 1: neighbouring warps meet on named barriers after a step, 0: the CTA
  // item scheduling: CTA b first runs the static run [b * static_items, (b + 1) *
  // static_items) (consecutive shots of mostly one tile, whose shot-independent
  // tables it keeps), then takes single items from the counter sched (zeroed before
  // the launch) after the static runs; sched == nullptr: a grid stride
  int* sched;
  int static_items;
  // sources
  const SrcNode* src;    // (nshots, nsrc_max) merged injection nodes
  int nsrc_max;
  const SrcTap* stap;    // nodes per (shot, tile), sorted by (thread, row, column)
  const int* stap_off;   // (nshots * ntiles + 1) offsets into stap
  int nsrow_max;         // staged source rows of the largest (shot, tile)
  const float* waveforms;
  int wave_len;
  // state (nshots, ny, pitch)
  const float* in_prev;
  const float* in_cur;
  float* out_prev;
  float* out_cur;
  // steps: FWD/REC n0 .. n0+nsteps-1, ADJ n0 .. n0-nsteps+1
  int n0, nsteps;
  // FWD
  float* traces;
  int nrx, nt;
  // REC / ADJ
  float* seg;
  long long seg_stride;  // elements between consecutive steps of the segment buffer
  int seg_base;          // step held in segment slot 0
  const float* residual;
  double* grad;
  double scale;          // adjoint: dt^2 / dy^2 (the stream holds Q = dy^2 lap), applied per pass
  // PML (pml != nullptr): tables, the face fields psi_x / psi_y in and out
  // (nshots, ny, pitch), and the per-CTA capacity of thread slots holding a
  // thread's face fields in shared memory
  const float* pml;
  const float* in_psx;
  const float* in_psy;
  float* out_psx;
  float* out_psy;
  int slot_cap;
};

// Several plans of one launch shape advanced by one launch (uneven batches).
struct TbGroup {
  const TbParams* params;  // (nplans) device array
  const int* item_off;     // (nplans + 1) prefix sums of tiles * shots
  int nplans, nitems;
};

// Dynamic shared-memory carve-up of the temporally blocked kernel; the host
// sizes the launch with the same function.
struct TbSmem {
  size_t coef, lap, g, xch, mur, tap, res, src, smask, sbase, pcol, prow, pxch, slots, nslot, total;
};

__host__ __device__ inline size_t tb_align16(size_t v) { return (v + 15) & ~size_t(15); }

__host__ __device__ inline TbSmem tb_smem_layout(int nw, int ky, int mode, int nrow_max,
                                                 int nrxl_max, int tmax, int adj_coef, int nsrow_max,
                                                 int slot_cap = 0) {
  TbSmem m;
  const size_t region = size_t(nw) * ky * RX * sizeof(float);
  size_t off = 0;
  // every mode keeps the region's coefficients in shared memory, except an
  // adjoint whose launch shape leaves no room (adj_coef = 0): it reads them
  // through L1 and shares the space with the next step's Laplacian tile, which
  // the adjoint streams in with cp.async
  m.coef = off;
  m.lap = off;
  off += region;
  if (mode == MODE_ADJ && adj_coef) {
    m.lap = off;
    off += region;
  }
  m.g = off;  // (the adjoint's gradient tile lives in tensor memory)
  m.xch = off; off += size_t(2) * nw * 2 * 32 * 16;
  // Mur table of an edge tile: k set and ratio set, each 2 region heights +
  // 2 region widths + 8 corner values
  m.mur = off; off += tb_align16(size_t(2) * (2 * size_t(nw) * ky + 2 * RX + 8) * sizeof(float));
  // tap stage: per step, the full 4-cell row of every (thread, band row) that holds
  // a receiver tap node (forward: recorded values; adjoint: injections, zero
  // where a row's cell has no tap)
  m.tap = off; off += size_t(tmax) * (nrow_max > 0 ? nrow_max : 1) * 4 * sizeof(float);
  m.res = off; if (mode == MODE_ADJ) off += tb_align16(size_t(nrxl_max > 0 ? nrxl_max : 1) * tmax * sizeof(float));
  // source stage: per step, the 4-cell rows holding this shot's injection nodes
  // (forward and recompute only)
  m.src = off; if (mode != MODE_ADJ) off += size_t(tmax) * (nsrow_max > 0 ? nsrow_max : 1) * 4 * sizeof(float);
  m.smask = off; off += size_t(nw) * 32 * sizeof(unsigned);
  m.sbase = off; off += size_t(nw) * 32 * sizeof(int);
  // PML grids (slot_cap > 0): the region's column and row tables (one row more,
  // for the face above the last band), the double-buffered exchange of each
  // band's first-row psi_y, and the thread slots (psi_x, psi_y of KY rows)
  m.pcol = m.prow = m.pxch = m.slots = m.nslot = off;
  if (slot_cap > 0) {
    off = tb_align16(off);
    m.pcol = off; off += size_t(PML_TABLES) * RX * sizeof(float);
    m.prow = off; off += tb_align16(size_t(PML_TABLES) * (size_t(nw) * ky + 1) * sizeof(float));
    m.pxch = off; off += size_t(2) * nw * 32 * 16;
    m.slots = off; off += size_t(slot_cap) * 2 * ky * 16;
    m.nslot = off; off += 16;
  }
  m.total = tb_align16(off);
  return m;
}

}  // namespace fdtd
