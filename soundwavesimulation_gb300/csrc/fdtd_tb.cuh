// Temporally blocked, shot-batched leapfrog kernel (forward, recompute, adjoint):
// the kernel templates, included by fdtd_tb.cu (grids with Mur edges) and
// fdtd_tb_pml.cu (grids with a PML layer), so that each family compiles on its own
// registers and the Mur kernels carry no PML code.
//
// One CTA works on one (tile, shot) item at a time, persistently. A tile is a
// region of 128 columns x (warps * KY) rows. Lane `l` of warp `w` keeps, in
// registers, columns 4l..4l+3 of rows w*KY..w*KY+KY-1 of the two live fields
// (u_old and u). A launch advances every region by `nsteps` leapfrog steps
// without touching HBM between steps:
//   - x-neighbours come from warp shuffles (the warp spans the whole region
//     width, so no shared memory is needed in x);
//   - y-neighbours inside a band stay in registers; the first and last row of
//     every band go through a double-buffered shared-memory exchange, after
//     which each neighbouring pair of warps meets on a named barrier (step_sync);
//   - the region carries a halo of at least nsteps+1 cells at every border that
//     is not a domain edge, so the cells a tile owns are still exact after the
//     last step (overlapped temporal blocking); owned cells partition the grid
//     and are the only ones written back;
//   - Mur edges and corners (fdtd2d/torch_backend.py:477-490), soft sources
//     (fdtd2d/torch_backend.py:517), the residual injection
//     (fdtd2d/torch_backend.py:563-580), the receiver gather
//     (fdtd2d/torch_backend.py:540-548), the per-step stencil value Q = dy^2 lap
//     of the forward field (recompute) and the imaging condition
//     (fdtd2d/torch_backend.py:583-598) are all applied inside the block:
//     receiver taps and source nodes as per-step shared-memory stages of whole
//     4-cell rows, Mur coefficients from a per-tile shared-memory table, the
//     adjoint's gradient tile in tensor memory (tcgen05) and its Q stream one
//     step ahead through cp.async;
//   - items are (tile, shot) pairs, costliest tiles first; the forward runs static
//     runs of consecutive items (reusing the tile's tables) and then takes items
//     from a per-launch counter, the recompute and adjoint a grid stride;
//   - each warp runs one of three loop variants per item: no edge work, the
//     compact edge form (edge rows at fixed band rows, whole-row Mur updates,
//     corners last) or the general one; the per-step loop of the common cases
//     stays small, which keeps it in the instruction cache.
// The stencil runs on cell pairs with the two-lane float32 instructions (the
// x-neighbour sums, whose operands straddle register pairs, are scalar); like
// the scalar helpers in fdtd_device.cuh every element is one IEEE
// round-to-nearest operation, so the values are bit-identical to the one-step
// kernels in fdtd_kernels.cu. `tb_group_kernel` runs the items of several plans
// (grids) in one launch.

#pragma once

#include "fdtd_device.cuh"
#include "fdtd_internal.h"

namespace fdtd {
namespace {

constexpr unsigned FULL = 0xffffffffu;

// Edge work of one warp for one item (warp-uniform). EK_EDGE is the compact
// form for the usual placements (row 0 at band row 0, row ny-1 at band row
// KY-1, column nx-1 not in column 0 of a lane); EK_ALL is the general form.
// Keeping the per-step loop of every common case small keeps it in the
// instruction cache.
constexpr int EK_NONE = 0, EK_EDGE = 1, EK_ALL = 2;
// EK_PML: a warp holding cells of a PML layer (PML grids have no Mur edges).
constexpr int EK_PML = 3;

struct Ctx {
  int tid, w, lane, nw, s;
  int cur_tile;             // the tile whose shot-independent tables shared memory holds (-1: none)
  int rx0, ry0, flags;
  int y0, xb;               // global row of this thread's r = 0, column of c = 0
  unsigned own_rows, own_cols;
  unsigned rfull;           // recompute: owned band rows whose 4-cell row it stores (it owns every
                            // column of the row that lies inside the grid)
  unsigned mask, smask;     // band rows holding receiver taps / source nodes
  unsigned rowvalid;        // band rows inside the domain (adjoint coefficient loads)
  int base, sbase;          // first staged tap row / source row of this thread
  const float* gcoef;       // global coefficients at (y0, xb) (adjoint)
  float* s_coef;
  float* s_lap;
  unsigned tm;              // adjoint: tensor-memory address of this thread's gradient tile
  float4* s_xch;
  float* s_mur;             // the tile's Mur table (edge tiles)
  float* s_tap;
  float* s_src;
  // PML grids
  const float* s_pcol;      // the region's column tables (PML_TABLES x RX)
  const float* s_prow;      // the region's row tables (PML_TABLES x (RY + 1))
  float4* s_pxch;           // first-row psi_y of every band, double-buffered
  float4* slot;             // this thread's psi_x rows [0, KY) and psi_y rows [KY, 2 KY), or null
};

// Stencil operand of one band row: the field itself in every mode (the adjoint
// is carried as w = coef l, so its update has the forward's form).
__device__ __forceinline__ float4 opval(const float (&v)[4]) {
  return make_float4(v[0], v[1], v[2], v[3]);
}

__device__ __forceinline__ float4 ldg4(const float* p) {
  return __ldg(reinterpret_cast<const float4*>(p));
}

// A state row, read once per item: not allocated in L1 (the 128 KB an item loads
// would otherwise evict the small tables every item reads; measured +0.3 % in the
// forward and +0.2 % in the gradient).
__device__ __forceinline__ float4 ldg4_once(const float* p) {
  float4 v;
  asm("ld.global.nc.L1::no_allocate.v4.f32 {%0, %1, %2, %3}, [%4];"
      : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
      : "l"(p));
  return v;
}

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}

__device__ __forceinline__ void cp_async4(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gmem) : "memory");
}

__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }

__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

// ---- tensor memory (TMEM) holds the adjoint's gradient tile
//
// 128 columns per CTA. Warp w reaches the TMEM lanes of quadrant w % 4 (lane l of
// the warp is TMEM lane 32 (w % 4) + l) and uses columns 4 KY (w / 4) ..
// 4 KY (w / 4) + 4 KY - 1: column 4 r + c holds cell (r, c) of the thread. The
// imaging read-modify-write thus runs through the tensor-memory datapath instead
// of the shared-memory pipe.
constexpr unsigned TM_COLS = 128;

__device__ __forceinline__ unsigned smem_u32(const void* ptr) {
  return (unsigned)__cvta_generic_to_shared(ptr);
}

__device__ __forceinline__ void tm_alloc(unsigned* dst) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)), "r"(TM_COLS)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tm_dealloc(unsigned base) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(base), "r"(TM_COLS) : "memory");
}

__device__ __forceinline__ void tm_fence_sync() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void tm_ld8(unsigned addr, unsigned (&v)[8]) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
               : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7])
               : "r"(addr)
               : "memory");
}

__device__ __forceinline__ void tm_st8(unsigned addr, const unsigned (&v)[8]) {
  asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"r"(addr),
               "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7])
               : "memory");
}

__device__ __forceinline__ void tm_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }
__device__ __forceinline__ void tm_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

// End of a step. Only the warps above and below read the rows a warp published,
// so with pair_sync each neighbouring pair (j, j+1) meets on its own named
// barrier j+1 (barrier 0 stays the CTA-wide __syncthreads): the pairs (2i, 2i+1)
// first, then (2i+1, 2i+2), so that no barrier waits on a chain of others. Warps
// d apart then drift by up to d steps instead of all waiting for the slowest one
// every step, which spreads the CTA's bursts of stencil arithmetic over time. The
// double-buffered exchange stays safe: a warp overwrites the buffer it published
// two steps earlier only after both neighbours met it at the end of the step
// that read it.
__device__ __forceinline__ void step_sync(const TbParams& p, const Ctx& x) {
  if (!p.pair_sync) {
    __syncthreads();
    return;
  }
  const int a = x.w | 1, b = (x.w + 1) & ~1;
  if (a < x.nw) asm volatile("bar.sync %0, 64;" ::"r"(a) : "memory");
  if (b >= 1 && b < x.nw) asm volatile("bar.sync %0, 64;" ::"r"(b) : "memory");
}

// Coefficients b = (c dt / dy)^2 of band row r: from the shared-memory copy of the region
// or, for an adjoint without room for it, through L1 from global memory; zero
// outside the domain.
template <int MODE, bool CS>
__device__ __forceinline__ float4 coefrow(const TbParams& p, const Ctx& x, const float4* coef4, int r) {
  if (MODE != MODE_ADJ || CS) return coef4[r * 32];
  if (!((x.rowvalid >> r) & 1u)) return make_float4(0.f, 0.f, 0.f, 0.f);
  return ldg4(x.gcoef + (long long)r * p.pitch);
}

// Streams Q(u^{n-1}) = dy^2 lap(u^{n-1}) of this thread's owned rows for adjoint
// step n into its slots of the shared-memory tile, all four columns of a row in one
// 16-byte copy (a column the thread does not own reads whatever the segment
// buffer holds there and is never flushed; xb + 3 < pitch since pitch is a
// multiple of 4).
template <int KY>
__device__ __forceinline__ void prefetch_lap(const TbParams& p, const Ctx& x, int n) {
  const float* sl = p.seg + (long long)(n - p.seg_base) * p.seg_stride +
                    ((long long)x.s * p.ny + x.y0) * p.pitch + x.xb;
  float* dst = x.s_lap + (x.w * KY) * RX + 4 * x.lane;
  if (x.own_rows == (1u << KY) - 1u) {  // warp-uniform: a band owned in full
#pragma unroll
    for (int r = 0; r < KY; ++r) cp_async16(dst + r * RX, sl + (long long)r * p.pitch);
  } else {
#pragma unroll
    for (int r = 0; r < KY; ++r)
      if ((x.own_rows >> r) & 1u) cp_async16(dst + r * RX, sl + (long long)r * p.pitch);
  }
  cp_async_commit();
}

// float32 -> float64 with integer instructions (exact for normal numbers and
// infinities; subnormal values, never reached by the imaging sums, become zero),
// which keeps the flush off GB300's narrow float64 pipe.
__device__ __forceinline__ double widen(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned e = (u >> 23) & 0xFFu;
  unsigned long long b = (unsigned long long)(u & 0x80000000u) << 32;
  if (e != 0u) b |= ((unsigned long long)(e == 0xFFu ? 0x7FFu : e + 896u) << 52) | ((unsigned long long)(u & 0x7FFFFFu) << 29);
  return __longlong_as_double((long long)b);
}

// One row pair of the imaging: v (the pair's gradient values from tensor memory) +=
// F rows r, r+1 times their Laplacian rows la, lb, all four columns.
template <int KY>
__device__ __forceinline__ void image_pair(const float (&F)[KY][4], int r, const float4& la, const float4& lb,
                                           unsigned (&v)[8]) {
  float2 g;
  g = __ffma2_rn(make_float2(F[r][0], F[r][1]), make_float2(la.x, la.y),
                 make_float2(__uint_as_float(v[0]), __uint_as_float(v[1])));
  v[0] = __float_as_uint(g.x); v[1] = __float_as_uint(g.y);
  g = __ffma2_rn(make_float2(F[r][2], F[r][3]), make_float2(la.z, la.w),
                 make_float2(__uint_as_float(v[2]), __uint_as_float(v[3])));
  v[2] = __float_as_uint(g.x); v[3] = __float_as_uint(g.y);
  g = __ffma2_rn(make_float2(F[r + 1][0], F[r + 1][1]), make_float2(lb.x, lb.y),
                 make_float2(__uint_as_float(v[4]), __uint_as_float(v[5])));
  v[4] = __float_as_uint(g.x); v[5] = __float_as_uint(g.y);
  g = __ffma2_rn(make_float2(F[r + 1][2], F[r + 1][3]), make_float2(lb.z, lb.w),
                 make_float2(__uint_as_float(v[6]), __uint_as_float(v[7])));
  v[6] = __float_as_uint(g.x); v[7] = __float_as_uint(g.y);
}

// Imaging of this thread's band: the gradient tile in tensor memory += F times the
// Laplacian tile that the previous step streamed into shared memory (cp.async).
// Row pairs are pipelined: the next pair's tensor-memory load is issued before the
// current pair's arithmetic and store, so one load is always in flight. Every pair
// is imaged, owned or not (a cell this thread does not own sums whatever its slot
// holds, and is never flushed). Warp-uniform: the caller checks own_rows.
template <int KY>
__device__ __forceinline__ void image_band(const Ctx& x, const float (&F)[KY][4]) {
  cp_async_wait_all();
  __syncwarp();  // the tensor-memory instructions need the whole warp converged
  tm_wait_st();
  const float4* l4 = reinterpret_cast<const float4*>(x.s_lap) + (x.w * KY) * 32 + x.lane;
  unsigned va[8], vb[8];  // gradient values of the even / odd row pairs
  tm_ld8(x.tm, va);
#pragma unroll
  for (int r = 0; r < KY; r += 2) {
    const float4 la = l4[r * 32];
    const float4 lb = l4[(r + 1) * 32];
    tm_wait_ld();
    // (the two buffers are named in separate branches, never selected by an
    // expression, so that they stay in registers)
    if ((r >> 1) & 1) {
      if (r + 2 < KY) tm_ld8(x.tm + 4 * (r + 2), va);
      image_pair<KY>(F, r, la, lb, vb);
      tm_st8(x.tm + 4 * r, vb);
    } else {
      if (r + 2 < KY) tm_ld8(x.tm + 4 * (r + 2), vb);
      image_pair<KY>(F, r, la, lb, va);
      tm_st8(x.tm + 4 * r, va);
    }
  }
}

// Mur edges and corners, in registers (plus shuffles across one lane boundary).
// The tiler places rows 0/1 and ny-2/ny-1 in one band and column 0 at lane 0, c = 0.
// Cells outside the domain need no per-step treatment: they are loaded as zero
// and their coef is zero, so in the forward they stay exactly zero
// (u+ = 2 * 0 - 0 + 0 * lap) and the zero-padded Laplacian
// the recompute stores is exact; in the adjoint their operand coef * l is zero,
// so whatever they hold never reaches a domain cell, and they are never written
// back.
// The Mur values of KY consecutive region rows (16-byte aligned in the table).
template <int KY>
__device__ __forceinline__ void load_rows(float (&v)[KY], const float* src) {
#pragma unroll
  for (int q = 0; q < KY / 4; ++q) {
    const float4 t = reinterpret_cast<const float4*>(src)[q];
    v[4 * q] = t.x; v[4 * q + 1] = t.y; v[4 * q + 2] = t.z; v[4 * q + 3] = t.w;
  }
}

// One Mur edge cell; with the ratio r = 1 (forward) murw reduces to mur exactly.
template <bool WF>
__device__ __forceinline__ float mur_edge(float r, float w_in, float k, float wn_in, float w_edge) {
  return WF ? murw(r, w_in, k, wn_in, w_edge) : mur(w_in, k, wn_in, w_edge);
}

// Left / right Mur column of one lane: edge column CE, inner column CI of the same
// lane, band rows rlo..rhi (all rows in the common case, without per-row tests).
template <int KY, bool WF, int CE, int CI>
__device__ __forceinline__ void mur_column(float (&P)[KY][4], const float (&C)[KY][4], const float* k,
                                           const float* ratio, int rlo, int rhi) {
  float kv[KY], rv[KY];
  load_rows<KY>(kv, k);
  if (WF) load_rows<KY>(rv, ratio);
  if (rlo <= 0 && rhi >= KY - 1) {
#pragma unroll
    for (int r = 0; r < KY; ++r)
      P[r][CE] = mur_edge<WF>(WF ? rv[r] : 1.0f, C[r][CI], kv[r], P[r][CI], C[r][CE]);
  } else {
#pragma unroll
    for (int r = 0; r < KY; ++r)
      if (r >= rlo && r <= rhi) P[r][CE] = mur_edge<WF>(WF ? rv[r] : 1.0f, C[r][CI], kv[r], P[r][CI], C[r][CE]);
  }
}

// Bottom / top Mur row RE of one lane from the inner row RI (columns 1 .. nx-2).
template <int KY, bool WF, int RE, int RI>
__device__ __forceinline__ void mur_row(float (&P)[KY][4], const float (&C)[KY][4], const float* k,
                                        const float* ratio, int xb, int nx) {
  const float4 kv = *reinterpret_cast<const float4*>(k);
  const float4 rv = WF ? *reinterpret_cast<const float4*>(ratio) : make_float4(1.f, 1.f, 1.f, 1.f);
  const float kk[4] = {kv.x, kv.y, kv.z, kv.w}, rr[4] = {rv.x, rv.y, rv.z, rv.w};
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    const float m = mur_edge<WF>(rr[c], C[RI][c], kk[c], P[RI][c], C[RE][c]);
    if (xb + c >= 1 && xb + c <= nx - 2) P[RE][c] = m;
  }
}

// mur_row at the runtime band row `re`, inner row re + DIR (compile-time dispatch).
template <int KY, bool WF, int DIR, int R = 0>
__device__ __forceinline__ void mur_row_at(float (&P)[KY][4], const float (&C)[KY][4], int re, const float* k,
                                           const float* ratio, int xb, int nx) {
  if constexpr (R + DIR >= 0 && R + DIR < KY) {
    if (re == R) {
      mur_row<KY, WF, R, R + DIR>(P, C, k, ratio, xb, nx);
      return;
    }
  }
  if constexpr (R + 1 < KY) mur_row_at<KY, WF, DIR, R + 1>(P, C, re, k, ratio, xb, nx);
}

// Mur row RE of one lane from the inner row RI on all four columns. The cells
// this also touches besides columns 1 .. nx-2 are corners (overwritten below)
// and padding columns (k = 0 and zero operands keep them zero).
template <int KY, bool WF, int RE, int RI>
__device__ __forceinline__ void mur_row_all(float (&P)[KY][4], const float (&C)[KY][4], const float* k,
                                            const float* ratio) {
  const float4 kv = *reinterpret_cast<const float4*>(k);
  const float4 rv = WF ? *reinterpret_cast<const float4*>(ratio) : make_float4(1.f, 1.f, 1.f, 1.f);
  P[RE][0] = mur_edge<WF>(rv.x, C[RI][0], kv.x, P[RI][0], C[RE][0]);
  P[RE][1] = mur_edge<WF>(rv.y, C[RI][1], kv.y, P[RI][1], C[RE][1]);
  P[RE][2] = mur_edge<WF>(rv.z, C[RI][2], kv.z, P[RI][2], C[RE][2]);
  P[RE][3] = mur_edge<WF>(rv.w, C[RI][3], kv.w, P[RI][3], C[RE][3]);
}

// Corner (band row R, lane column CE) as the average of the x-direction Mur from
// column CI and the y-direction Mur from band row RN; kC[ci] / kC[4 + ci] are the
// corner's kx / ky (ratios rofs further on for the w-form).
template <int KY, bool WF, int R, int RN, int CE, int CI>
__device__ __forceinline__ void corner(float (&P)[KY][4], const float (&C)[KY][4], const float* kC, int ci,
                                       int rofs) {
  const float fx = mur_edge<WF>(WF ? kC[rofs + ci] : 1.0f, C[R][CI], kC[ci], P[R][CI], C[R][CE]);
  const float fy = mur_edge<WF>(WF ? kC[rofs + 4 + ci] : 1.0f, C[RN][CE], kC[4 + ci], P[RN][CE], C[R][CE]);
  P[R][CE] = corner_avg(fx, fy);
}

// Right-edge work in lane L1 for the column c1 = 1, 2, 3 holding nx-1 (inner
// column c1 - 1 in the same lane): the column over every band row, then the
// corners of the rows the band holds.
template <int KY, bool WF, int CE>
__device__ __forceinline__ void right_fast(float (&P)[KY][4], const float (&C)[KY][4], const float* kR,
                                           const float* kC, int rofs, bool bot, bool top) {
  mur_column<KY, WF, CE, CE - 1>(P, C, kR, kR + rofs, 0, KY - 1);
  if (bot) corner<KY, WF, 0, 1, CE, CE - 1>(P, C, kC, 1, rofs);
  if (top) corner<KY, WF, KY - 1, KY - 2, CE, CE - 1>(P, C, kC, 3, rofs);
}

// EK_EDGE: Mur rows on whole lane rows, columns on every band row, then the
// corners, which overwrite the four corner cells the rows and columns also
// touched (the reference's order: rows and columns from the same field, corners
// from their updated neighbours).
template <int KY, bool WF>
__device__ __forceinline__ void boundary_fast(float (&P)[KY][4], const float (&C)[KY][4],
                                              const TbParams& p, const Ctx& x) {
  const int ry = x.nw * KY;
  const float* kL = x.s_mur;
  const float* kR = kL + ry;
  const float* kB = kR + ry;
  const float* kT = kB + RX;
  const float* kC = kT + RX;
  const int rofs = 2 * ry + 2 * RX + 8;
  const int lr0 = x.w * KY, lc0 = 4 * x.lane;
  const bool bot = (x.flags & TF_BOTTOM) && x.y0 == 0;                // warp-uniform
  const bool top = (x.flags & TF_TOP) && x.y0 + KY == p.ny;           // warp-uniform
  if (bot) mur_row_all<KY, WF, 0, 1>(P, C, kB + lc0, kB + rofs + lc0);
  if (top) mur_row_all<KY, WF, KY - 1, KY - 2>(P, C, kT + lc0, kT + rofs + lc0);
  if ((x.flags & TF_LEFT) && x.lane == 0) {
    mur_column<KY, WF, 0, 1>(P, C, kL + lr0, kL + rofs + lr0, 0, KY - 1);
    if (bot) corner<KY, WF, 0, 1, 0, 1>(P, C, kC, 0, rofs);
    if (top) corner<KY, WF, KY - 1, KY - 2, 0, 1>(P, C, kC, 2, rofs);
  }
  if (x.flags & TF_RIGHT) {
    const int lx1 = p.nx - 1 - x.rx0;
    if (x.lane == (lx1 >> 2)) {
      const int c1 = lx1 & 3;   // 1, 2 or 3 in this variant
      if (c1 == 3) right_fast<KY, WF, 3>(P, C, kR + lr0, kC, rofs, bot, top);
      else if (c1 == 2) right_fast<KY, WF, 2>(P, C, kR + lr0, kC, rofs, bot, top);
      else right_fast<KY, WF, 1>(P, C, kR + lr0, kC, rofs, bot, top);
    }
  }
}

template <int KY, bool WF>
__device__ __forceinline__ void boundary(float (&P)[KY][4], const float (&C)[KY][4],
                                         const TbParams& p, const Ctx& x) {
  const int nx = p.nx, ny = p.ny;
  // the tile's Mur table in shared memory (filled per item, local indices):
  // k left / right per region row, bottom / top per region column, corner kx[4],
  // ky[4]; for the w-form adjoint the same layout again holds the ratios
  // coef_edge / coef_inner that scale the inner values (1 otherwise)
  const int ry = x.nw * KY;
  const float* kL = x.s_mur;
  const float* kR = kL + ry;
  const float* kB = kR + ry;
  const float* kT = kB + RX;
  const float* kC = kT + RX;
  const int rofs = 2 * ry + 2 * RX + 8;
  auto R = [&](const float* k, int j) { return WF ? k[rofs + j] : 1.0f; };
  const int lr0 = x.w * KY;      // region row of band row 0
  const int lc0 = 4 * x.lane;    // region column of c = 0
  const int rb = -x.y0;          // band row of global row 0
  const int rt = ny - 1 - x.y0;  // band row of global row ny-1
  const bool has_bot = (x.flags & TF_BOTTOM) && rb >= 0 && rb + 1 < KY;   // warp-uniform
  const bool has_top = (x.flags & TF_TOP) && rt >= 1 && rt < KY;          // warp-uniform
  // bottom / top Mur rows on the columns 1 .. nx-2 of this lane (row 0 is band
  // row 0 of the first warp whenever the region starts at row 0, as the tiler
  // places it; other positions take the general form)
  if (has_bot) {
    if (rb == 0) mur_row<KY, WF, 0, 1>(P, C, kB + lc0, kB + rofs + lc0, x.xb, nx);
    else mur_row_at<KY, WF, 1>(P, C, rb, kB + lc0, kB + rofs + lc0, x.xb, nx);
  }
  if (has_top) mur_row_at<KY, WF, -1>(P, C, rt, kT + lc0, kT + rofs + lc0, x.xb, nx);
  // rows 1 .. ny-2 of the band take the left / right Mur update
  const int rlo = 1 - x.y0, rhi = ny - 2 - x.y0;
  if ((x.flags & TF_LEFT) && x.lane == 0) mur_column<KY, WF, 0, 1>(P, C, kL + lr0, kL + rofs + lr0, rlo, rhi);
  if (x.flags & TF_RIGHT) {
    const int lx1 = nx - 1 - x.rx0;
    const int L1 = lx1 >> 2, c1 = lx1 & 3;   // tile-uniform
    // Column nx-2 sits in the same lane (c1 >= 1) or in column 3 of the previous
    // lane (c1 == 0: one shuffle pair per row, executed by the whole warp). The
    // edge rows are updated first, so the corners below see updated values.
    if (c1 == 0) {
#pragma unroll
      for (int r = 0; r < KY; ++r) {
        const float su = __shfl_up_sync(FULL, C[r][3], 1);
        const float sn = __shfl_up_sync(FULL, P[r][3], 1);
        if (x.lane == L1 && r >= rlo && r <= rhi)
          P[r][0] = mur_edge<WF>(R(kR, lr0 + r), su, kR[lr0 + r], sn, C[r][0]);
      }
    } else if (x.lane == L1) {
      if (c1 == 3) mur_column<KY, WF, 3, 2>(P, C, kR + lr0, kR + rofs + lr0, rlo, rhi);
      else if (c1 == 2) mur_column<KY, WF, 2, 1>(P, C, kR + lr0, kR + rofs + lr0, rlo, rhi);
      else mur_column<KY, WF, 1, 0>(P, C, kR + lr0, kR + rofs + lr0, rlo, rhi);
    }
    if (has_bot || has_top) {  // corners (0, nx-1) and (ny-1, nx-1)
#pragma unroll
      for (int r = 0; r < KY; ++r) {
        const bool bot = has_bot && r == rb;
        const bool top = has_top && r == rt;
        if (bot || top) {  // warp-uniform
          float su = 0.f, sn = 0.f;
          if (c1 == 0) {
            su = __shfl_up_sync(FULL, C[r][3], 1);
            sn = __shfl_up_sync(FULL, P[r][3], 1);
          }
          if (x.lane == L1) {
            const int rn = bot ? (r + 1 < KY ? r + 1 : r) : (r >= 1 ? r - 1 : r);
            const int ci = bot ? 1 : 3;
#pragma unroll
            for (int c = 0; c < 4; ++c) {
              if (c == c1) {
                const float uin = (c == 0) ? su : C[r][c > 0 ? c - 1 : 0];
                const float nin = (c == 0) ? sn : P[r][c > 0 ? c - 1 : 0];
                const float fx = murw(R(kC, ci), uin, kC[ci], nin, C[r][c]);
                const float fy = murw(R(kC, 4 + ci), C[rn][c], kC[4 + ci], P[rn][c], C[r][c]);
                P[r][c] = corner_avg(fx, fy);
              }
            }
          }
        }
      }
    }
  }
  if ((x.flags & TF_LEFT) && x.lane == 0 && (has_bot || has_top)) {  // corners (0, 0), (ny-1, 0)
#pragma unroll
    for (int r = 0; r < KY; ++r) {
      const bool bot = has_bot && r == rb;
      const bool top = has_top && r == rt;
      if (bot || top) {
        const int rn = bot ? (r + 1 < KY ? r + 1 : r) : (r >= 1 ? r - 1 : r);
        const int ci = bot ? 0 : 2;
        const float fx = murw(R(kC, ci), C[r][1], kC[ci], P[r][1], C[r][0]);
        const float fy = murw(R(kC, 4 + ci), C[rn][0], kC[4 + ci], P[rn][0], C[r][0]);
        P[r][0] = corner_avg(fx, fy);
      }
    }
  }
}

template <int KY, int MODE, int EK, bool CS>
__device__ __forceinline__ void substep(float (&P)[KY][4], float (&C)[KY][4],
                                        const TbParams& p, const Ctx& x, int k) {
  const int n = (MODE == MODE_ADJ) ? p.n0 - k : p.n0 + k;
  const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);
  const float4* xin = x.s_xch + (k & 1) * x.nw * 64;
  float4* xout = x.s_xch + ((k + 1) & 1) * x.nw * 64;
  const float4* coef4 = reinterpret_cast<const float4*>(x.s_coef) + (x.w * KY) * 32 + x.lane;
  // Paired-lane (f32x2) arithmetic: every element is rounded once, exactly like the
  // scalar helpers of fdtd_device.cuh (nbrq / lapq / leap), so the values stay
  // bit-identical to the one-step kernels while one instruction updates two cells.
  const float2 R2 = make_float2(p.ratio, p.ratio), Q2 = make_float2(p.qdiag, p.qdiag);
  const float2 TWO2 = make_float2(2.0f, 2.0f);

  // ---- stencil over the band, rolling the row above / below
  float4 prv = (x.w > 0) ? xin[(x.w - 1) * 64 + 32 + x.lane] : zero4;
  const float4 below = (x.w < x.nw - 1) ? xin[(x.w + 1) * 64 + x.lane] : zero4;
  float4 cur = opval(C[0]);
  // Column 0 and column nx-1 are always overwritten by the Mur update, so only
  // the recompute, which stores lap(u) itself, needs the zero outside the domain.
  const bool lzero = EK != EK_NONE && mode_stream(MODE) && x.lane == 0 && x.rx0 == 0;
  const bool rzero = EK != EK_NONE && mode_stream(MODE) && x.lane == 31 && (x.rx0 + RX >= p.nx);
  float* segrow = nullptr;
  if (mode_stream(MODE)) {
    segrow = p.seg + (long long)(n - p.seg_base) * p.seg_stride +
             ((long long)x.s * p.ny + x.y0) * p.pitch + x.xb;
  }
#pragma unroll
  for (int r = 0; r < KY; ++r) {
    const float4 nxt = (r + 1 < KY) ? opval(C[r + 1]) : below;
    float lft = __shfl_up_sync(FULL, cur.w, 1);
    float rgt = __shfl_down_sync(FULL, cur.x, 1);
    if (lzero) lft = 0.f;
    if (rzero) rgt = 0.f;
    // nbrq / lapq / leap of fdtd_device.cuh on cell pairs (0,1) and (2,3): the
    // stencil Q = dy^2 lap against the coefficient b = (c dt / dy)^2. The
    // left + right sums are scalar: their operands (lft, c0), (c1, c2), (c3, rgt)
    // straddle the register pairs, and a paired add would first need them
    // copied into place (more instructions than the four scalar adds).
    const float2 udA = __fadd2_rn(make_float2(prv.x, prv.y), make_float2(nxt.x, nxt.y));
    const float2 udB = __fadd2_rn(make_float2(prv.z, prv.w), make_float2(nxt.z, nxt.w));
    const float2 lrA = make_float2(__fadd_rn(lft, cur.y), __fadd_rn(cur.x, cur.z));
    const float2 lrB = make_float2(__fadd_rn(cur.y, cur.w), __fadd_rn(cur.z, rgt));
    const float2 nA = __ffma2_rn(lrA, R2, udA);
    const float2 nB = __ffma2_rn(lrB, R2, udB);
    {
      const float4 co = coefrow<MODE, CS>(p, x, coef4, r);
      const float2 lA = __ffma2_rn(make_float2(cur.x, cur.y), Q2, nA);
      const float2 lB = __ffma2_rn(make_float2(cur.z, cur.w), Q2, nB);
      if (mode_stream(MODE)) {
        // Q = dy^2 lap (the adjoint's flush scale carries the 1 / dy^2): each
        // owned row in one predicated 16-byte store
        if ((x.rfull >> r) & 1u) *reinterpret_cast<float4*>(segrow) = make_float4(lA.x, lA.y, lB.x, lB.y);
        segrow += p.pitch;
      }
      const float2 tA = __ffma2_rn(TWO2, make_float2(cur.x, cur.y), make_float2(-P[r][0], -P[r][1]));
      const float2 tB = __ffma2_rn(TWO2, make_float2(cur.z, cur.w), make_float2(-P[r][2], -P[r][3]));
      const float2 uA = __ffma2_rn(make_float2(co.x, co.y), lA, tA);
      const float2 uB = __ffma2_rn(make_float2(co.z, co.w), lB, tB);
      P[r][0] = uA.x;
      P[r][1] = uA.y;
      P[r][2] = uB.x;
      P[r][3] = uB.y;
    }
    prv = cur;
    cur = nxt;
  }

  // ---- injection before the boundary update
  if (MODE != MODE_ADJ) {
    if (x.smask) {
      // source injection: whole staged rows, zero where a cell holds no node
      const float4* inj = reinterpret_cast<const float4*>(x.s_src) + k * p.nsrow_max + x.sbase;
      int slot = 0;
#pragma unroll
      for (int r = 0; r < KY; ++r) {
        if ((x.smask >> r) & 1u) {
          const float4 v = inj[slot];
          P[r][0] = inj_add(P[r][0], v.x);
          P[r][1] = inj_add(P[r][1], v.y);
          P[r][2] = inj_add(P[r][2], v.z);
          P[r][3] = inj_add(P[r][3], v.w);
          ++slot;
        }
      }
    }
  } else if (x.mask) {
    // residual injection: whole staged rows, zero where a cell holds no tap
    const float4* inj = reinterpret_cast<const float4*>(x.s_tap) + k * p.nrow_max + x.base;
    int slot = 0;
#pragma unroll
    for (int r = 0; r < KY; ++r) {
      if ((x.mask >> r) & 1u) {
        const float4 v = inj[slot];
        P[r][0] = inj_add(P[r][0], v.x);
        P[r][1] = inj_add(P[r][1], v.y);
        P[r][2] = inj_add(P[r][2], v.z);
        P[r][3] = inj_add(P[r][3], v.w);
        ++slot;
      }
    }
  }

  // ---- Mur edges and corners, zero outside the domain
  if (EK == EK_EDGE) boundary_fast<KY, MODE == MODE_ADJ>(P, C, p, x);
  if (EK == EK_ALL) boundary<KY, MODE == MODE_ADJ>(P, C, p, x);

  // ---- receiver taps (forward) / imaging (adjoint)
  if (mode_traces(MODE) && x.mask) {
    // stage every band row that holds a tap node, all four cells of it
    float4* rec = reinterpret_cast<float4*>(x.s_tap) + k * p.nrow_max + x.base;
    int slot = 0;
#pragma unroll
    for (int r = 0; r < KY; ++r) {
      if ((x.mask >> r) & 1u) {
        rec[slot] = make_float4(P[r][0], P[r][1], P[r][2], P[r][3]);
        ++slot;
      }
    }
  }
  if (MODE == MODE_ADJ && x.own_rows) {  // warp-uniform: the tensor-memory ops are warp-wide
    if (n >= 1) {
      image_band<KY>(x, P);
    }
    if (x.own_cols && k + 1 < p.nsteps && n - 1 >= 1) prefetch_lap<KY>(p, x, n - 1);
  }

  // ---- publish the band's first and last rows for the next step
  xout[x.w * 64 + x.lane] = opval(P[0]);
  xout[x.w * 64 + 32 + x.lane] = opval(P[KY - 1]);
  step_sync(p, x);
}

// psi_y (new) on the bottom faces of one lane row: decay of the old value plus
// (sigma_x - sigma_y,face) beta_y (u - u_below), per column.
__device__ __forceinline__ float4 pml_face_y(const float4& po, const float4& sxc, float syf, float ayf, float byf,
                                             const float4& u, const float4& ub) {
  return make_float4(pml_face(ayf, po.x, sxc.x, syf, byf, __fsub_rn(u.x, ub.x)),
                     pml_face(ayf, po.y, sxc.y, syf, byf, __fsub_rn(u.y, ub.y)),
                     pml_face(ayf, po.z, sxc.z, syf, byf, __fsub_rn(u.z, ub.z)),
                     pml_face(ayf, po.w, sxc.w, syf, byf, __fsub_rn(u.w, ub.w)));
}

// One step of a warp holding PML layer cells: the face fields psi_x, psi_y (this
// thread's shared-memory slot; none: zero), the PML update factors, and no Mur
// edges (a PML grid ends in a rigid wall behind the layer: u and psi are zero
// beyond it). psi_x on a lane's right face is the next lane's left-face value of
// the same step (a shuffle); psi_y on a band's top face is recomputed from the
// next band's first row and its published old psi_y, so one step barrier
// still suffices. Sources, receivers, the recompute's Laplacian and the imaging
// are as in substep; where sigma = 0 the values are bit for bit the plain ones.
template <int KY, int MODE, bool CS>
__device__ __forceinline__ void substep_pml(float (&P)[KY][4], float (&C)[KY][4], const TbParams& p,
                                            const Ctx& x, int k) {
  const int n = (MODE == MODE_ADJ) ? p.n0 - k : p.n0 + k;
  const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);
  const float4* xin = x.s_xch + (k & 1) * x.nw * 64;
  float4* xout = x.s_xch + ((k + 1) & 1) * x.nw * 64;
  const float4* pin = x.s_pxch + (k & 1) * x.nw * 32;
  float4* pout = x.s_pxch + ((k + 1) & 1) * x.nw * 32;
  const float4* coef4 = reinterpret_cast<const float4*>(x.s_coef) + (x.w * KY) * 32 + x.lane;
  const float2 R2 = make_float2(p.ratio, p.ratio), Q2 = make_float2(p.qdiag, p.qdiag);
  const float4 sxc = reinterpret_cast<const float4*>(x.s_pcol)[x.lane];
  const float4 sxf = reinterpret_cast<const float4*>(x.s_pcol + RX)[x.lane];
  const float4 axf = reinterpret_cast<const float4*>(x.s_pcol + 2 * RX)[x.lane];
  const float4 bxf = reinterpret_cast<const float4*>(x.s_pcol + 3 * RX)[x.lane];
  const int RYp = x.nw * KY + 1;
  const float* syc = x.s_prow;
  const float* syf = x.s_prow + RYp;
  const float* ayf = x.s_prow + 2 * RYp;
  const float* byf = x.s_prow + 3 * RYp;
  const int r0 = x.w * KY;
  float4* slot = x.slot;
  const bool lzero = x.lane == 0 && x.rx0 == 0;          // grid column 0: zero beyond
  const bool rzero = x.lane == 31 && x.rx0 + RX >= p.nx;  // the grid's right side: zero beyond

  float4 prv = (x.w > 0) ? xin[(x.w - 1) * 64 + 32 + x.lane] : zero4;
  const float4 below = (x.w < x.nw - 1) ? xin[(x.w + 1) * 64 + x.lane] : zero4;
  const float4 psy_up = (x.w < x.nw - 1) ? pin[(x.w + 1) * 32 + x.lane] : zero4;
  float4 cur = opval(C[0]);
  float4 pyb = pml_face_y(slot ? slot[KY] : zero4, sxc, syf[r0], ayf[r0], byf[r0], cur, prv);
  const float4 pyb0 = pyb;
  float* segrow = nullptr;
  if (mode_stream(MODE)) {
    segrow = p.seg + (long long)(n - p.seg_base) * p.seg_stride +
             ((long long)x.s * p.ny + x.y0) * p.pitch + x.xb;
  }
#pragma unroll
  for (int r = 0; r < KY; ++r) {
    const float4 nxt = (r + 1 < KY) ? opval(C[r + 1]) : below;
    float lft = __shfl_up_sync(FULL, cur.w, 1);
    float rgt = __shfl_down_sync(FULL, cur.x, 1);
    if (lzero) lft = 0.f;
    if (rzero) rgt = 0.f;
    const float sy = syc[r0 + r];
    const float4 pxo = slot ? slot[r] : zero4;
    const float4 pxl = make_float4(pml_face(axf.x, pxo.x, sy, sxf.x, bxf.x, __fsub_rn(cur.x, lft)),
                                   pml_face(axf.y, pxo.y, sy, sxf.y, bxf.y, __fsub_rn(cur.y, cur.x)),
                                   pml_face(axf.z, pxo.z, sy, sxf.z, bxf.z, __fsub_rn(cur.z, cur.y)),
                                   pml_face(axf.w, pxo.w, sy, sxf.w, bxf.w, __fsub_rn(cur.w, cur.z)));
    float pxr3 = __shfl_down_sync(FULL, pxl.x, 1);
    if (rzero) pxr3 = 0.f;
    const int rn = r0 + r + 1;
    const float4 pyo = (r + 1 < KY) ? (slot ? slot[KY + r + 1] : zero4) : psy_up;
    const float4 pyt = pml_face_y(pyo, sxc, syf[rn], ayf[rn], byf[rn], nxt, cur);
    if (slot) {
      slot[r] = pxl;
      slot[KY + r] = pyb;
    }
    // the stencil Q = dy^2 lap exactly as substep computes it
    const float2 udA = __fadd2_rn(make_float2(prv.x, prv.y), make_float2(nxt.x, nxt.y));
    const float2 udB = __fadd2_rn(make_float2(prv.z, prv.w), make_float2(nxt.z, nxt.w));
    const float2 lrA = make_float2(__fadd_rn(lft, cur.y), __fadd_rn(cur.x, cur.z));
    const float2 lrB = make_float2(__fadd_rn(cur.y, cur.w), __fadd_rn(cur.z, rgt));
    const float2 nA = __ffma2_rn(lrA, R2, udA);
    const float2 nB = __ffma2_rn(lrB, R2, udB);
    const float2 lA = __ffma2_rn(make_float2(cur.x, cur.y), Q2, nA);
    const float2 lB = __ffma2_rn(make_float2(cur.z, cur.w), Q2, nB);
    if (mode_stream(MODE)) {
      // Q = dy^2 lap, as substep stores it
      if ((x.rfull >> r) & 1u) *reinterpret_cast<float4*>(segrow) = make_float4(lA.x, lA.y, lB.x, lB.y);
      segrow += p.pitch;
    }
    const float4 co = coefrow<MODE, CS>(p, x, coef4, r);
    float A, M;
    pml_factors(sxc.x, sy, A, M);
    P[r][0] = pml_leap(cur.x, P[r][0], co.x, A, M, lA.x, pml_div(pxl.x, pxl.y, pyb.x, pyt.x));
    pml_factors(sxc.y, sy, A, M);
    P[r][1] = pml_leap(cur.y, P[r][1], co.y, A, M, lA.y, pml_div(pxl.y, pxl.z, pyb.y, pyt.y));
    pml_factors(sxc.z, sy, A, M);
    P[r][2] = pml_leap(cur.z, P[r][2], co.z, A, M, lB.x, pml_div(pxl.z, pxl.w, pyb.z, pyt.z));
    pml_factors(sxc.w, sy, A, M);
    P[r][3] = pml_leap(cur.w, P[r][3], co.w, A, M, lB.y, pml_div(pxl.w, pxr3, pyb.w, pyt.w));
    pyb = pyt;
    prv = cur;
    cur = nxt;
  }

  // ---- injection (sources in the forward / recompute, the residual in the adjoint)
  if (MODE != MODE_ADJ) {
    if (x.smask) {
      const float4* inj = reinterpret_cast<const float4*>(x.s_src) + k * p.nsrow_max + x.sbase;
      int sl = 0;
#pragma unroll
      for (int r = 0; r < KY; ++r) {
        if ((x.smask >> r) & 1u) {
          const float4 v = inj[sl];
          P[r][0] = inj_add(P[r][0], v.x);
          P[r][1] = inj_add(P[r][1], v.y);
          P[r][2] = inj_add(P[r][2], v.z);
          P[r][3] = inj_add(P[r][3], v.w);
          ++sl;
        }
      }
    }
  } else if (x.mask) {
    const float4* inj = reinterpret_cast<const float4*>(x.s_tap) + k * p.nrow_max + x.base;
    int sl = 0;
#pragma unroll
    for (int r = 0; r < KY; ++r) {
      if ((x.mask >> r) & 1u) {
        const float4 v = inj[sl];
        P[r][0] = inj_add(P[r][0], v.x);
        P[r][1] = inj_add(P[r][1], v.y);
        P[r][2] = inj_add(P[r][2], v.z);
        P[r][3] = inj_add(P[r][3], v.w);
        ++sl;
      }
    }
  }
  if (mode_traces(MODE) && x.mask) {
    float4* rec = reinterpret_cast<float4*>(x.s_tap) + k * p.nrow_max + x.base;
    int sl = 0;
#pragma unroll
    for (int r = 0; r < KY; ++r) {
      if ((x.mask >> r) & 1u) {
        rec[sl] = make_float4(P[r][0], P[r][1], P[r][2], P[r][3]);
        ++sl;
      }
    }
  }
  if (MODE == MODE_ADJ && x.own_rows) {
    if (n >= 1) image_band<KY>(x, P);
    if (x.own_cols && k + 1 < p.nsteps && n - 1 >= 1) prefetch_lap<KY>(p, x, n - 1);
  }

  // ---- publish the band's first and last rows and its first-row psi_y
  xout[x.w * 64 + x.lane] = opval(P[0]);
  xout[x.w * 64 + 32 + x.lane] = opval(P[KY - 1]);
  pout[x.w * 32 + x.lane] = pyb0;
  step_sync(p, x);
}

template <int KY>
__device__ __forceinline__ void store_state(const TbParams& p, const Ctx& x,
                                            const float (&prev)[KY][4], const float (&cur)[KY][4]) {
  if (!x.own_rows || !x.own_cols) return;
  const long long base = ((long long)x.s * p.ny + x.y0) * p.pitch + x.xb;
#pragma unroll
  for (int r = 0; r < KY; ++r) {
    if ((x.own_rows >> r) & 1u) {
      float* dp = p.out_prev + base + (long long)r * p.pitch;
      float* dc = p.out_cur + base + (long long)r * p.pitch;
      if (x.own_cols == 0xFu) {
        *reinterpret_cast<float4*>(dp) = make_float4(prev[r][0], prev[r][1], prev[r][2], prev[r][3]);
        *reinterpret_cast<float4*>(dc) = make_float4(cur[r][0], cur[r][1], cur[r][2], cur[r][3]);
      } else {
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          if ((x.own_cols >> c) & 1u) {
            dp[c] = prev[r][c];
            dc[c] = cur[r][c];
          }
        }
      }
    }
  }
}

// The item's two state fields, this thread's band rows (zero outside the domain;
// padding columns: see zero_padding). Issued at the start of the item so that
// their latency overlaps the table setup.
template <int KY, bool LATE_PAD>
__device__ __forceinline__ void load_state(const TbParams& p, const Ctx& x, float (&P)[KY][4], float (&C)[KY][4]) {
  const long long sbase = (long long)x.s * p.ny * p.pitch;
#pragma unroll
  for (int r = 0; r < KY; ++r) {
    const int yy = x.y0 + r;
    float4 a = make_float4(0.f, 0.f, 0.f, 0.f), b = a;
    if (yy >= 0 && yy < p.ny && x.xb < p.pitch) {
      a = ldg4_once(p.in_prev + sbase + (long long)yy * p.pitch + x.xb);
      b = ldg4_once(p.in_cur + sbase + (long long)yy * p.pitch + x.xb);
    }
    P[r][0] = a.x; P[r][1] = a.y; P[r][2] = a.z; P[r][3] = a.w;
    C[r][0] = b.x; C[r][1] = b.y; C[r][2] = b.z; C[r][3] = b.w;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      if (!LATE_PAD && x.xb + c >= p.nx) { P[r][c] = 0.f; C[r][c] = 0.f; }
    }
  }
}

// Padding columns (x >= nx) start every item at zero whatever the buffer holds
// there. With LATE_PAD (every mode but the adjoint) this runs at the end of the item
// setup, not in load_state: overwriting a register that a load is still filling
// waits for the load, which would hold the whole setup behind the state's latency
// (the forward measured 2.3 % faster; the adjoint, at its register limit, spilled
// more and kept the early form).
template <int KY>
__device__ __forceinline__ void zero_padding(const TbParams& p, const Ctx& x, float (&P)[KY][4],
                                             float (&C)[KY][4]) {
  if (x.xb + 3 < p.nx) return;
#pragma unroll
  for (int r = 0; r < KY; ++r) {
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      if (x.xb + c >= p.nx) { P[r][c] = 0.f; C[r][c] = 0.f; }
    }
  }
}

// Pulls the state rows of this thread in item `item` (the CTA's next one) into
// L2 while the current item computes.
template <int KY>
__device__ __forceinline__ void prefetch_state(const TbParams& p, const Ctx& x, int item) {
  const int ti = item / p.nshots;
  const int s = item - ti * p.nshots;
  const TbTile& t = p.tiles[ti];
  const int y0 = t.ry0 + x.w * KY, xb = t.rx0 + 4 * x.lane;
  if (xb >= p.pitch) return;
  const long long sbase = (long long)s * p.ny * p.pitch;
#pragma unroll
  for (int r = 0; r < KY; ++r) {
    const int yy = y0 + r;
    if (yy >= 0 && yy < p.ny) {
      const long long o = sbase + (long long)yy * p.pitch + xb;
      asm volatile("prefetch.global.L2 [%0];" ::"l"(p.in_prev + o));
      asm volatile("prefetch.global.L2 [%0];" ::"l"(p.in_cur + o));
    }
  }
}

// The T steps of one item; the item setup has published the band's first and
// last rows and met the whole CTA.
template <int KY, int MODE, int EK, bool CS>
__device__ __forceinline__ void run_item(const TbParams& p, const Ctx& x, float (&P)[KY][4], float (&C)[KY][4]) {
  if (MODE == MODE_ADJ && x.own_rows && x.own_cols && p.n0 >= 1) prefetch_lap<KY>(p, x, p.n0);

  for (int k = 0; k < p.nsteps; k += 2) {
    if constexpr (EK == EK_PML) {
      substep_pml<KY, MODE, CS>(P, C, p, x, k);
      if (k + 1 < p.nsteps) substep_pml<KY, MODE, CS>(C, P, p, x, k + 1);
    } else {
      substep<KY, MODE, EK, CS>(P, C, p, x, k);
      if (k + 1 < p.nsteps) substep<KY, MODE, EK, CS>(C, P, p, x, k + 1);
    }
  }
  // the item's end reads every warp's staged taps; with CTA-wide step barriers
  // the last step's barrier is this one. Past it no thread reads a shared buffer
  // that the next item's setup writes before its own CTA barrier, so an item
  // needs no barrier after its traces and stores.
  if (p.pair_sync) __syncthreads();
  if (p.nsteps & 1) {
    store_state<KY>(p, x, C, P);
  } else {
    store_state<KY>(p, x, P, C);
  }
}

// Binds the context's shared-memory carve-up for the launch parameters `p`.
template <int KY, int MODE>
__device__ __forceinline__ void bind_ctx(const TbParams& p, Ctx& x, unsigned char* smem) {
  const TbSmem L = tb_smem_layout(p.nwarps, KY, MODE, p.nrow_max, p.nrxl_max, p.tmax, p.adj_coef, p.nsrow_max,
                                  p.slot_cap);
  x.nw = p.nwarps;
  x.s_pcol = reinterpret_cast<const float*>(smem + L.pcol);
  x.s_prow = reinterpret_cast<const float*>(smem + L.prow);
  x.s_pxch = reinterpret_cast<float4*>(smem + L.pxch);
  x.slot = nullptr;
  x.s_coef = reinterpret_cast<float*>(smem + L.coef);
  x.s_lap = reinterpret_cast<float*>(smem + L.lap);
  x.s_xch = reinterpret_cast<float4*>(smem + L.xch);
  x.s_mur = reinterpret_cast<float*>(smem + L.mur);
  x.s_tap = reinterpret_cast<float*>(smem + L.tap);
  x.s_src = reinterpret_cast<float*>(smem + L.src);
}

// The loop variant of one warp for one item; CS: the coefficient tile is in shared
// memory (every mode but an adjoint without room for it), a compile-time choice (a
// kernel of its own) so that the step loop has no per-row branch on it.
template <int KY, int MODE, bool PML, bool CS>
__device__ __forceinline__ void dispatch_item(const TbParams& p, const Ctx& x, float (&P)[KY][4], float (&C)[KY][4],
                                              int ek) {
  if constexpr (PML) {
    if (ek == EK_PML) {
      run_item<KY, MODE, EK_PML, CS>(p, x, P, C);
      return;
    }
  }
  if (ek == EK_NONE) run_item<KY, MODE, EK_NONE, CS>(p, x, P, C);
  else if (ek == EK_EDGE) run_item<KY, MODE, EK_EDGE, CS>(p, x, P, C);
  else if (ek == EK_ALL) run_item<KY, MODE, EK_ALL, CS>(p, x, P, C);
}

// One (tile, shot) item: load, T steps, store, traces / gradient flush; `next` is
// the CTA's next item of the same launch (or -1), whose state is prefetched; with
// dyn_next it is read from there after the item's first CTA barrier. The region's
// coefficient tile, Mur table and PML tables are kept from the previous item when
// it was the same tile (consecutive shots of a static run).
template <int KY, int MODE, bool PML, bool CS>
__device__ __forceinline__ void run_one(const TbParams& p, Ctx& x, unsigned char* smem, int item, int next,
                                        const int* dyn_next = nullptr) {
  const int nw = p.nwarps;
  const int nthr = nw * 32;
  const TbSmem L = tb_smem_layout(nw, KY, MODE, p.nrow_max, p.nrxl_max, p.tmax, p.adj_coef, p.nsrow_max,
                                  p.slot_cap);
  float* s_res = reinterpret_cast<float*>(smem + L.res);
  unsigned* s_smask = reinterpret_cast<unsigned*>(smem + L.smask);
  int* s_sbase = reinterpret_cast<int*>(smem + L.sbase);
  {
    const int ti = item / p.nshots;
    const int s = item - ti * p.nshots;
    const TbTile t = p.tiles[ti];
    // (the forward only: the recompute and adjoint, at their register limit, deal
    // their items with a grid stride, where consecutive items are other tiles)
    const bool same_tile = MODE == MODE_FWD && ti == x.cur_tile;  // CTA-uniform
    if (MODE == MODE_FWD) x.cur_tile = ti;
    x.s = s;
    x.rx0 = t.rx0;
    x.ry0 = t.ry0;
    x.flags = t.flags;
    x.y0 = t.ry0 + x.w * KY;
    x.xb = t.rx0 + 4 * x.lane;
    x.own_rows = 0;
    x.rowvalid = 0;
#pragma unroll
    for (int r = 0; r < KY; ++r) {
      const int yy = x.y0 + r;
      if (yy >= t.oy0 && yy < t.oy1) x.own_rows |= 1u << r;
      if (yy >= 0 && yy < p.ny && x.xb < p.pitch) x.rowvalid |= 1u << r;
    }
    x.gcoef = p.coef + (long long)x.y0 * p.pitch + x.xb;
    x.own_cols = 0;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const int xx = x.xb + c;
      if (xx >= t.ox0 && xx < t.ox1) x.own_cols |= 1u << c;
    }
    // (padding columns beyond nx count as owned: no other tile writes them, and
    // the adjoint never reads them back into the gradient; gradient plans place
    // every other ownership boundary between lanes)
    {
      unsigned ext = x.own_cols;
#pragma unroll
      for (int c = 0; c < 4; ++c)
        if (x.xb + c >= p.nx) ext |= 1u << c;
      x.rfull = (x.own_cols && ext == 0xFu) ? x.own_rows : 0u;
    }
    float P[KY][4], C[KY][4];
    constexpr bool LATE_PAD = MODE != MODE_ADJ;
    load_state<KY, LATE_PAD>(p, x, P, C);
    if (next >= 0) prefetch_state<KY>(p, x, next);

    // coefficients of the region (zero outside the domain; the padding columns of
    // coef are zero in memory) and, below, the Mur table. The forward issues them
    // as asynchronous copies, all in flight together with the state loads and
    // awaited before the barrier that precedes the first step (measured 5 %
    // faster); the recompute and adjoint, at their register limit, load them
    // through registers.
    constexpr bool ASYNC_FILL = MODE == MODE_FWD;
#pragma unroll
    for (int r = 0; r < KY; ++r) {
      if (!same_tile && (MODE != MODE_ADJ || p.adj_coef)) {
        float4* dst = reinterpret_cast<float4*>(x.s_coef) + (x.w * KY + r) * 32 + x.lane;
        if (ASYNC_FILL && ((x.rowvalid >> r) & 1u)) {
          cp_async16(dst, x.gcoef + (long long)r * p.pitch);
        } else {
          float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
          if ((x.rowvalid >> r) & 1u) v = ldg4(x.gcoef + (long long)r * p.pitch);
          *dst = v;
        }
      }
    }
    if (MODE == MODE_ADJ) {  // cleared gradient tile in tensor memory
      const unsigned z[8] = {0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u};
      __syncwarp();
      tm_wait_st();
#pragma unroll
      for (int c = 0; c < 4 * KY; c += 8) tm_st8(x.tm + c, z);
    }
    bool pml_tile = false;
    if constexpr (PML) pml_tile = p.pml && (t.flags & TF_PML);
    x.slot = nullptr;
    if (PML && pml_tile) {
      // the region's PML tables (zero outside the grid; one row more than the
      // region for the face above the last band), an empty slot counter and
      // cleared psi_y exchange buffers
      const int RYp = nw * KY + 1;
      float* pc = const_cast<float*>(x.s_pcol);
      float* pr = const_cast<float*>(x.s_prow);
      if (!same_tile) {
        for (int i = x.tid; i < PML_TABLES * RX; i += nthr) {
          const int tbl = i / RX, gx = t.rx0 + i - tbl * RX;
          pc[i] = (gx >= 0 && gx < p.nx) ? __ldg(p.pml + tbl * p.nx + gx) : 0.f;
        }
        for (int i = x.tid; i < PML_TABLES * RYp; i += nthr) {
          const int tbl = i / RYp, gy = t.ry0 + i - tbl * RYp;
          pr[i] = (gy >= 0 && gy < p.ny) ? __ldg(p.pml + PML_TABLES * p.nx + tbl * p.ny + gy) : 0.f;
        }
      }
      for (int i = x.tid; i < 2 * nw * 32; i += nthr) x.s_pxch[i] = make_float4(0.f, 0.f, 0.f, 0.f);
      if (x.tid == 0) *reinterpret_cast<int*>(smem + L.nslot) = 0;
    }
    if ((t.flags & TF_MUR) && !same_tile) {
      // the tile's Mur table: left / right k per region row, bottom / top per
      // region column, corner kx / ky; the adjoint also copies the ratio set
      const int ry = nw * KY, len = 2 * ry + 2 * RX + 8, glen = 2 * p.ny + 2 * p.nx + 8;
      for (int i = x.tid; i < len * (MODE == MODE_ADJ ? 2 : 1); i += nthr) {
        const int set = (MODE == MODE_ADJ && i >= len) ? 1 : 0, j = i - set * len;
        const float* g = p.mur + set * glen;
        const float* src = nullptr;
        if (j < 2 * ry) {
          const int side = j >= ry, gy = t.ry0 + j - side * ry;
          if (gy >= 0 && gy < p.ny) src = g + side * p.ny + gy;
        } else if (j < 2 * ry + 2 * RX) {
          const int side = j >= 2 * ry + RX, gx = t.rx0 + j - 2 * ry - side * RX;
          if (gx >= 0 && gx < p.nx) src = g + 2 * p.ny + side * p.nx + gx;
        } else {
          src = g + 2 * p.ny + 2 * p.nx + (j - 2 * ry - 2 * RX);
        }
        if (ASYNC_FILL && src) cp_async4(x.s_mur + i, src);
        else x.s_mur[i] = src ? __ldg(src) : 0.f;
      }
    }
    // this shot's injection nodes inside the region (sorted by thread, row, column)
    const int so = (MODE != MODE_ADJ) ? __ldg(p.stap_off + s * p.ntiles + ti) : 0;
    const int ns = (MODE != MODE_ADJ) ? __ldg(p.stap_off + s * p.ntiles + ti + 1) - so : 0;
    s_smask[x.tid] = 0u;  // (read back by this thread only; other threads' atomics follow a barrier)
    s_sbase[x.tid] = 0x7fffffff;
    if (MODE != MODE_ADJ && ns > 0) {
      // staged source rows start at zero: cells without a node add nothing
      const int nrows = p.stap[so + ns - 1].srow + 1;
      for (int i = x.tid; i < p.nsteps * nrows; i += nthr) {
        const int k = i / nrows, j = i - k * nrows;
        reinterpret_cast<float4*>(x.s_src)[k * p.nsrow_max + j] = make_float4(0.f, 0.f, 0.f, 0.f);
      }
    }
    if (MODE == MODE_ADJ) {
      // staged injection rows start at zero: cells without a tap add nothing
      for (int i = x.tid; i < p.nsteps * t.nrow; i += nthr) {
        const int k = i / t.nrow, j = i - k * t.nrow;
        reinterpret_cast<float4*>(x.s_tap)[k * p.nrow_max + j] = make_float4(0.f, 0.f, 0.f, 0.f);
      }
      for (int i = x.tid; i < t.nrxl * p.nsteps; i += nthr) {
        const int j = i / p.nsteps, k = i - j * p.nsteps;
        const int rg = __ldg(p.rxl + t.rxl_off + j);
        s_res[j * p.tmax + k] = __ldg(p.residual + ((long long)s * p.nrx + rg) * p.nt + (p.n0 - k));
      }
    }
    // the cleared stages, residual samples and PML tables before their cooperative
    // fills below (items without sources, injections or PML cells skip it)
    if (MODE == MODE_ADJ || ns > 0 || pml_tile) __syncthreads();
    bool pml_warp = false;
    if (PML && pml_tile) {
      // a thread holding a layer cell (sigma_x > 0 in one of its columns or
      // sigma_y > 0 in one of its rows) takes a slot for its face fields and loads
      // them; its whole warp runs the PML step
      bool layer = false;
#pragma unroll
      for (int c = 0; c < 4; ++c) layer |= x.s_pcol[4 * x.lane + c] > 0.f;
#pragma unroll
      for (int r = 0; r < KY; ++r) layer |= x.s_prow[x.w * KY + r] > 0.f;
      pml_warp = __any_sync(FULL, layer);
      if (layer) {
        const int sl = atomicAdd(reinterpret_cast<int*>(smem + L.nslot), 1);
        if (sl < p.slot_cap) {  // the planner sizes slot_cap for the largest tile
          x.slot = reinterpret_cast<float4*>(smem + L.slots) + (size_t)sl * 2 * KY;
          const long long sb = (long long)x.s * p.ny * p.pitch;
#pragma unroll
          for (int r = 0; r < KY; ++r) {
            const int yy = x.y0 + r;
            float4 a = make_float4(0.f, 0.f, 0.f, 0.f), b = a;
            if (yy >= 0 && yy < p.ny && x.xb < p.pitch) {
              a = ldg4_once(p.in_psx + sb + (long long)yy * p.pitch + x.xb);
              b = ldg4_once(p.in_psy + sb + (long long)yy * p.pitch + x.xb);
            }
            x.slot[r] = a;
            x.slot[KY + r] = b;
          }
          // the first step's old psi_y of this band's first row, for the band below
          // (the exchange buffer the first step reads; a barrier follows)
          x.s_pxch[x.w * 32 + x.lane] = x.slot[KY];
        }
      }
    }
    // per thread: which band rows hold source nodes, and the first staged row;
    // the source values of every step go to the stage
    for (int i = x.tid; i < ns; i += nthr) {
      const SrcTap st = p.stap[so + i];
      atomicOr(&s_smask[st.packed >> 8], 1u << ((st.packed & 255) >> 2));
      atomicMin(&s_sbase[st.packed >> 8], st.srow);
    }
    for (int i = x.tid; i < ns * p.nsteps; i += nthr) {
      const int e = i / p.nsteps, k = i - e * p.nsteps;
      const SrcTap st = p.stap[so + e];
      const SrcNode sn = p.src[(long long)s * p.nsrc_max + st.node];
      const int nstep = p.n0 + k;
      float acc = 0.f;
#pragma unroll
      for (int q = 0; q < SRC_C; ++q) {
        if (sn.wave[q] >= 0) {
          const float v = (nstep < p.wave_len) ? __ldg(p.waveforms + (long long)sn.wave[q] * p.wave_len + nstep) : 0.f;
          acc = inj_acc(acc, sn.w[q], v);
        }
      }
      x.s_src[(k * p.nsrow_max + st.srow) * 4 + (st.packed & 3)] = acc;
    }
    if (MODE == MODE_ADJ) {
      for (int i = x.tid; i < t.ntap * p.nsteps; i += nthr) {
        const int ti2 = i / p.nsteps, k = i - ti2 * p.nsteps;
        const TbTap& tp = p.taps[t.tap_off + ti2];
        float acc = 0.f;
#pragma unroll
        for (int q = 0; q < TAP_C; ++q) {
          const int rl = tp.rloc[q];
          if (rl >= 0) acc = inj_acc(acc, tp.w[q], s_res[rl * p.tmax + k]);
        }
        // the adjoint is carried as w = coef * l: scale the injection by the node's coef
        const int pt = tp.packed >> 8, pb = tp.packed & 255;
        const int gy = t.ry0 + (pt >> 5) * KY + (pb >> 2), gx = t.rx0 + (pt & 31) * 4 + (pb & 3);
        x.s_tap[(k * p.nrow_max + tp.srow) * 4 + (pb & 3)] =
            __fmul_rn(__ldg(p.coef + (long long)gy * p.pitch + gx), acc);
      }
    }
    // this thread's band rows holding receiver tap nodes and its first staged tap
    // row (shot-independent, from the plan), and the band's first and last rows
    // for the first step
    const int2 tmk = __ldg(reinterpret_cast<const int2*>(p.tmask) + (long long)ti * nthr + x.tid);
    if (LATE_PAD) zero_padding<KY>(p, x, P, C);
    x.s_xch[x.w * 64 + x.lane] = opval(C[0]);
    x.s_xch[x.w * 64 + 32 + x.lane] = opval(C[KY - 1]);
    if (ASYNC_FILL) {  // the coefficient and Mur table copies
      cp_async_commit();
      cp_async_wait_all();
    }
    __syncthreads();
    if (dyn_next) {
      const int nx_item = *dyn_next;
      if (nx_item < p.ntiles * p.nshots) prefetch_state<KY>(p, x, nx_item);
    }
    x.mask = (unsigned)tmk.x;
    x.base = tmk.y;
    x.smask = s_smask[x.tid];
    x.sbase = s_sbase[x.tid];

    // Edge code only in warps with edge cells: every warp of a tile holding the
    // left or right edge (column 0 / nx-1 and the padding columns sit in every
    // band), only the warps holding row 0 or row ny-1 otherwise. Warps of one CTA
    // may take different variants: all pass the same per-step barriers.
    const bool row_b = (t.flags & TF_BOTTOM) && x.y0 <= 0 && x.y0 + KY > 0;
    const bool row_t = (t.flags & TF_TOP) && x.y0 <= p.ny - 1 && x.y0 + KY > p.ny - 1;
    const bool cols = t.flags & (TF_LEFT | TF_RIGHT);
    const bool fast = (!row_b || x.y0 == 0) && (!row_t || x.y0 + KY == p.ny) && !(row_b && row_t) &&
                      (!(t.flags & TF_RIGHT) || ((p.nx - 1 - t.rx0) & 3) != 0);
    const int ek = pml_warp ? EK_PML : (!row_b && !row_t && !cols) ? EK_NONE : fast ? EK_EDGE : EK_ALL;
    dispatch_item<KY, MODE, PML, CS>(p, x, P, C, ek);

    if (PML && x.slot && x.own_rows && x.own_cols) {
      // the face fields of the owned cells (cells without a slot hold zero there,
      // which the buffers keep from their initial clearing)
      const long long sb = ((long long)x.s * p.ny + x.y0) * p.pitch + x.xb;
#pragma unroll
      for (int r = 0; r < KY; ++r) {
        if ((x.own_rows >> r) & 1u) {
          const float4 a = x.slot[r], b = x.slot[KY + r];
          float* dx_ = p.out_psx + sb + (long long)r * p.pitch;
          float* dy_ = p.out_psy + sb + (long long)r * p.pitch;
          if (x.own_cols == 0xFu) {
            *reinterpret_cast<float4*>(dx_) = a;
            *reinterpret_cast<float4*>(dy_) = b;
          } else {
            const float av[4] = {a.x, a.y, a.z, a.w}, bv[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
            for (int c = 0; c < 4; ++c) {
              if ((x.own_cols >> c) & 1u) {
                dx_[c] = av[c];
                dy_[c] = bv[c];
              }
            }
          }
        }
      }
    }
    if (mode_traces(MODE)) {
      // receiver traces of the owned receivers, nsteps contiguous samples each
      for (int i = x.tid; i < t.nrec * p.nsteps; i += nthr) {
        const int j = i / p.nsteps, k = i - j * p.nsteps;
        const TbRec& rc = p.recs[t.rec_off + j];
        const float* v = x.s_tap + (long long)k * p.nrow_max * 4;
        const float smp = gather4(v[rc.slot[0]], v[rc.slot[1]], v[rc.slot[2]], v[rc.slot[3]],
                                  rc.w[0], rc.w[1], rc.w[2], rc.w[3]);
        p.traces[((long long)s * p.nrx + rc.rg) * p.nt + p.n0 + k] = smp;
      }
    }
    if (MODE == MODE_ADJ && x.own_rows) {  // warp-uniform: tensor-memory loads are warp-wide
      __syncwarp();
      tm_wait_st();
#pragma unroll
      for (int r0 = 0; r0 < KY; r0 += 2) {
        if (!((x.own_rows >> r0) & 3u)) continue;
        unsigned v[8];
        __syncwarp();
        tm_ld8(x.tm + 4 * r0, v);
        tm_wait_ld();
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const int r = r0 + h;
          if (!x.own_cols || !((x.own_rows >> r) & 1u)) continue;
          // the tile summed w * Q over the launch's steps (w = coef * l): the
          // cross-item sum is float64 (the widening is exact and takes integer
          // instructions, the sum is an L2 atomic), and the scale dt^2 / dy^2 and
          // the division by coef wait for the end of the pass (once per cell)
          double* gd = p.grad + (long long)(x.y0 + r) * p.pitch + x.xb;
#pragma unroll
          for (int c = 0; c < 4; ++c)
            if ((x.own_cols >> c) & 1u) atomicAdd(gd + c, widen(__uint_as_float(v[4 * h + c])));
        }
      }
    }
  }
}

// The adjoint's tensor-memory columns: allocated by warp 0 at kernel start and
// freed by it at the end; thread address of the gradient tile into x.tm.
template <int KY, int MODE>
__device__ __forceinline__ unsigned tm_begin(Ctx& x, unsigned* slot) {
  if (MODE != MODE_ADJ) return 0;
  if (x.w == 0) tm_alloc(slot);
  tm_fence_sync();
  const unsigned base = *slot;
  x.tm = base + ((unsigned)(32 * (x.w & 3)) << 16) + (unsigned)(4 * KY * (x.w >> 2));
  return base;
}

template <int MODE>
__device__ __forceinline__ void tm_end(const Ctx& x, unsigned base) {
  if (MODE != MODE_ADJ) return;
  __syncwarp();
  tm_wait_st();
  tm_fence_sync();
  if (x.w == 0) tm_dealloc(base);
}

template <int KY, int MODE, int MAXT, bool PML, bool CS>
__global__ void __launch_bounds__(MAXT, 1) tb_kernel(const TbParams p) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ unsigned tm_slot;
  Ctx x;
  x.tid = threadIdx.x;
  x.w = x.tid >> 5;
  x.lane = x.tid & 31;
  bind_ctx<KY, MODE>(p, x, smem);
  x.cur_tile = -1;
  const unsigned tm_base = tm_begin<KY, MODE>(x, &tm_slot);
  const int nitems = p.ntiles * p.nshots;
  // Items are (tile, shot) pairs with shots varying fastest, the costliest tiles
  // first. Each CTA runs a static run of consecutive items (mostly shots of one
  // tile, whose coefficient tile and Mur table it keeps), then takes single items
  // from a counter until none is left, so that CTAs whose runs were cheap take
  // more and the launch ends within about one item of its mean. The next dynamic
  // item is fetched by thread 0 at the start of the current one and read by all
  // threads after that item's barriers (double-buffered).
  // (one call site of run_one: the item code is inlined once)
  __shared__ int s_dyn[2];
  constexpr bool DYN = MODE == MODE_FWD;  // see run_one
  const int S = (DYN && p.sched) ? p.static_items : 0;
  const int s0 = (int)blockIdx.x * S, s1 = min(s0 + S, nitems);
  const int d0 = min((int)gridDim.x * S, nitems);  // first dynamically dealt item
  int par = 0;
  int item = (int)blockIdx.x;
  if (DYN && p.sched) {
    item = s0 < s1 ? s0 : -1;
    if (item < 0) {
      if (x.tid == 0) s_dyn[0] = d0 + atomicAdd(p.sched, 1);
      __syncthreads();
      item = s_dyn[0];
      par = 1;
    }
  }
  while (item < nitems) {
    int next = -1;
    const int* dyn = nullptr;
    if (!DYN || !p.sched) {
      next = item + (int)gridDim.x < nitems ? item + (int)gridDim.x : -1;
    } else if (item + 1 < s1) {
      next = item + 1;
    } else {
      if (x.tid == 0) s_dyn[par] = d0 + atomicAdd(p.sched, 1);
      dyn = &s_dyn[par];
    }
    run_one<KY, MODE, PML, CS>(p, x, smem, item, next, dyn);
    if (!DYN || !p.sched) {
      item += (int)gridDim.x;
    } else if (!dyn) {
      ++item;
    } else {
      item = s_dyn[par];
      par ^= 1;
    }
  }
  tm_end<MODE>(x, tm_base);
}

// Several plans (grids) of one launch shape in one launch: the items of plan i
// are [item_off[i], item_off[i+1]); a CTA copies the parameters of the plan of
// its current item into shared memory when the plan changes. CS: every plan of the
// group keeps its coefficient tile in shared memory (reading it through L1 serves
// any plan).
template <int KY, int MODE, int MAXT, bool CS>
__global__ void __launch_bounds__(MAXT, 1) tb_group_kernel(const TbGroup g) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ __align__(16) TbParams sp;
  __shared__ unsigned tm_slot;
  Ctx x;
  x.tid = threadIdx.x;
  x.w = x.tid >> 5;
  x.lane = x.tid & 31;
  const unsigned tm_base = tm_begin<KY, MODE>(x, &tm_slot);
  int cur = -1;
  for (int item = blockIdx.x; item < g.nitems; item += gridDim.x) {
    int pi = 0;
    while (pi + 1 < g.nplans && item >= __ldg(g.item_off + pi + 1)) ++pi;
    if (pi != cur) {
      __syncthreads();
      const int* src = reinterpret_cast<const int*>(g.params + pi);
      int* dst = reinterpret_cast<int*>(&sp);
      for (int i = x.tid; i < (int)(sizeof(TbParams) / sizeof(int)); i += blockDim.x) dst[i] = __ldg(src + i);
      __syncthreads();
      bind_ctx<KY, MODE>(sp, x, smem);
      x.cur_tile = -1;
      cur = pi;
    }
    run_one<KY, MODE, false, CS>(sp, x, smem, item - __ldg(g.item_off + pi), -1);
  }
  tm_end<MODE>(x, tm_base);
}

template <int KY, int MODE, int MAXT, bool PML, bool CS>
cudaError_t configure_one(size_t smem) {
  static size_t configured_smem = 0;  // per device it is the same binary; raise only
  if (smem > configured_smem) {
    cudaError_t e = cudaFuncSetAttribute(tb_kernel<KY, MODE, MAXT, PML, CS>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    configured_smem = smem;
  }
  return cudaSuccess;
}

template <int KY, int MODE, int MAXT, bool PML, bool CS>
cudaError_t launch_one(const TbParams& p, int grid, size_t smem, cudaStream_t st) {
  cudaError_t e = configure_one<KY, MODE, MAXT, PML, CS>(smem);
  if (e != cudaSuccess) return e;
  tb_kernel<KY, MODE, MAXT, PML, CS><<<grid, p.nwarps * 32, smem, st>>>(p);
  return cudaGetLastError();
}

// One mode at one shape; the adjoint has a kernel with its coefficient tile in
// shared memory and one that reads it through L1.
template <int KY, int MODE, int MAXT, bool PML>
cudaError_t launch_fixed(const TbParams& p, int grid, size_t smem, cudaStream_t st) {
  if constexpr (MODE == MODE_ADJ) {
    if (!p.adj_coef) return launch_one<KY, MODE, MAXT, PML, false>(p, grid, smem, st);
  }
  return launch_one<KY, MODE, MAXT, PML, true>(p, grid, smem, st);
}

template <int KY, int MODE, int MAXT, bool PML>
cudaError_t configure_fixed(size_t smem) {
  cudaError_t e = configure_one<KY, MODE, MAXT, PML, true>(smem);
  if constexpr (MODE == MODE_ADJ) {
    if (e == cudaSuccess) e = configure_one<KY, MODE, MAXT, PML, false>(smem);
  }
  return e;
}

// The four launch shapes: KY = 8 rows per lane with at most 12 warps (168
// registers per thread) or 16 warps (128 registers); KY = 4 with at most 16 warps
// (128 registers) or 32 warps (64 registers). One mode per instantiation, so that
// the modes compile in translation units of their own, in parallel.
template <int MODE, bool PML>
cudaError_t launch_shape(const TbParams& p, int ky, int grid, size_t smem, cudaStream_t st) {
  if (ky == 8) {
    if (p.nwarps <= 12) return launch_fixed<8, MODE, 384, PML>(p, grid, smem, st);
    return launch_fixed<8, MODE, 512, PML>(p, grid, smem, st);
  }
  if (p.nwarps <= 16) return launch_fixed<4, MODE, 512, PML>(p, grid, smem, st);
  return launch_fixed<4, MODE, 1024, PML>(p, grid, smem, st);
}

template <int MODE, bool PML>
cudaError_t configure_shape(int ky, int nwarps, size_t smem) {
  if (ky == 8) {
    if (nwarps <= 12) return configure_fixed<8, MODE, 384, PML>(smem);
    return configure_fixed<8, MODE, 512, PML>(smem);
  }
  if (nwarps <= 16) return configure_fixed<4, MODE, 512, PML>(smem);
  return configure_fixed<4, MODE, 1024, PML>(smem);
}

template <int KY, int MODE, int MAXT, bool CS>
cudaError_t group_one(const TbGroup& g, int nwarps, int grid, size_t smem, cudaStream_t st) {
  static size_t configured_smem = 0;
  if (smem > configured_smem) {
    cudaError_t e = cudaFuncSetAttribute(tb_group_kernel<KY, MODE, MAXT, CS>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    configured_smem = smem;
  }
  tb_group_kernel<KY, MODE, MAXT, CS><<<grid, nwarps * 32, smem, st>>>(g);
  return cudaGetLastError();
}

template <int KY, int MODE, int MAXT>
cudaError_t group_fixed(const TbGroup& g, int nwarps, bool adj_coef, int grid, size_t smem, cudaStream_t st) {
  if constexpr (MODE == MODE_ADJ) {
    if (!adj_coef) return group_one<KY, MODE, MAXT, false>(g, nwarps, grid, smem, st);
  }
  return group_one<KY, MODE, MAXT, true>(g, nwarps, grid, smem, st);
}

template <int MODE>
cudaError_t group_shape(const TbGroup& g, int ky, int nwarps, bool adj_coef, int grid, size_t smem,
                        cudaStream_t st) {
  if (ky == 8) {
    if (nwarps <= 12) return group_fixed<8, MODE, 384>(g, nwarps, adj_coef, grid, smem, st);
    return group_fixed<8, MODE, 512>(g, nwarps, adj_coef, grid, smem, st);
  }
  if (nwarps <= 16) return group_fixed<4, MODE, 512>(g, nwarps, adj_coef, grid, smem, st);
  return group_fixed<4, MODE, 1024>(g, nwarps, adj_coef, grid, smem, st);
}

}  // namespace

// Entry points of the translation units (one per family and mode group).
cudaError_t tb_launch_adj(const TbParams& p, int ky, int grid, size_t smem, cudaStream_t st);
cudaError_t tb_configure_adj(int ky, int nwarps, size_t smem);
cudaError_t tb_group_launch_adj(const TbGroup& g, int ky, int nwarps, bool adj_coef, int grid, size_t smem,
                                cudaStream_t st);
cudaError_t tb_launch_pml(const TbParams& p, int ky, int mode, int grid, size_t smem, cudaStream_t st);
cudaError_t tb_configure_pml(int ky, int mode, int nwarps, size_t smem);
cudaError_t tb_launch_pml_adj(const TbParams& p, int ky, int grid, size_t smem, cudaStream_t st);
cudaError_t tb_configure_pml_adj(int ky, int nwarps, size_t smem);

}  // namespace fdtd
