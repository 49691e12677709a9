// Host runtime of the engine: tiling, tap and source tables, checkpoint
// schedule, workspace layout, the time-loop executors and the C ABI.

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <string>
#include <utility>
#include <vector>

#include "../../include/fdtd_gb300.h"
#include "fdtd_internal.h"

namespace fdtd {

static thread_local std::string g_error;

void set_error(const std::string& msg) { g_error = msg; }

int32_t fail(int32_t code, const std::string& msg) {
  set_error(msg);
  return code;
}

int32_t cuda_fail(cudaError_t e, const char* what) {
  return fail(FDTD_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

namespace {

constexpr size_t ALIGN = 256;
// 227 KB opt-in shared memory per CTA, less what the kernels declare statically
// (the tensor-memory slot and the dynamic item buffers, 16 bytes; 64 reserved)
constexpr size_t SMEM_LIMIT = 232448 - TB_STATIC_SMEM;

size_t align_up(size_t v) { return (v + ALIGN - 1) / ALIGN * ALIGN; }

struct AxisTile {
  int origin, own0, own1, flags;  // flags: 1 low edge, 2 high edge, 4 outside cells
};

bool band_ok(int n, int origin, int region, int band) {
  if (band <= 1) return true;
  const int end = origin + region;
  if (origin <= 0 && 0 < end) {
    const int l = -origin;
    if (l % band == band - 1) return false;  // row 0 and row 1 would sit in different bands
  }
  if (origin <= n - 1 && n - 1 < end) {
    const int l = n - 1 - origin;
    if (l % band == 0) return false;  // row n-1 and row n-2 would sit in different bands
  }
  return true;
}

int floor_align(int v, int a) {
  if (a <= 1) return v;
  return (v >= 0) ? (v / a) * a : -(((-v) + a - 1) / a) * a;
}

// Greedy 1-D tiling; see fdtd_tile_axis in the public header.
std::string tile_axis(int n, int region, int align, int halo, int band, std::vector<AxisTile>& out) {
  out.clear();
  if (n < 4) return "grid axis must have at least 4 cells";
  if (region <= 2 * halo + 1) return "region too small for the temporal halo";
  int own0 = 0;
  while (own0 < n) {
    int origin = (own0 == 0) ? 0 : floor_align(own0 - halo, align);
    if (origin < 0 && align > 1) origin = 0;
    int tries = 0;
    while (!band_ok(n, origin, region, band)) {
      origin -= (align > 1 ? align : 1);
      if (++tries > 64) return "no region placement satisfies the band constraint";
    }
    if (band > 1 && origin > 0 && origin + region >= n) {
      // the last region: move it down (more overlap) until row n-1 is the last
      // row of its band, if it still reaches n, so that the kernel's compact edge
      // loop applies to the band holding row n-1
      int o = origin;
      while (o > 0 && (n - 1 - o) % band != band - 1) o -= (align > 1 ? align : 1);
      if (o > 0 && o + region >= n && band_ok(n, o, region, band)) origin = o;
    }
    const int end = origin + region;
    int own1 = (end >= n) ? n : end - halo;
    if (origin > 0 && own0 < origin + halo) return "tiler produced an unsafe low border";
    if (own1 <= own0) return "region too small to make progress";
    AxisTile t;
    t.origin = origin;
    t.own0 = own0;
    t.own1 = own1;
    t.flags = (origin <= 0 ? 1 : 0) | (end >= n ? 2 : 0) | ((origin < 0 || end > n) ? 4 : 0);
    out.push_back(t);
    own0 = own1;
    if (out.size() > 100000) return "too many tiles";
  }
  return "";
}

}  // namespace
}  // namespace fdtd

using namespace fdtd;

struct fdtd_plan {
  fdtd_problem prob;
  fdtd_tuning tun;
  int for_gradient = 0;
  int ky = 8, nw = 16, tmax = 12, RY = 128;
  std::vector<TbTile> tiles;
  std::vector<TbTap> taps;
  std::vector<TbMask> tmask;  // (tiles, threads): tap rows and first staged row per thread
  std::vector<int> rxl;
  std::vector<TbRec> recs;
  std::vector<SrcNode> src;       // (n_shots, nsrc_max) merged nodes
  std::vector<int> nsrc;
  std::vector<SrcTap> stap;       // per (shot, tile) nodes inside the region
  std::vector<int> stap_off;      // (n_shots * n_tiles + 1)
  int nsrc_max = 1, nsrow_max = 0;
  int nrow_max = 0, nrxl_max = 0;
  int adj_coef = 0;
  // gradient plans: the last `kept` checkpoint segments' stencil streams are written
  // by the forward (MODE_FWDQ) and kept, so the adjoint recomputes only the others
  int kept = 0;
  int pair_sync = 0;
  int ckpt_every = 0, nseg = 1;
  size_t field_elems = 0;
  // workspace offsets
  size_t o_tiles = 0, o_taps = 0, o_tmask = 0, o_rxl = 0, o_recs = 0, o_src = 0, o_stap = 0, o_stap_off = 0;
  size_t o_state[2][2] = {{0, 0}, {0, 0}};
  size_t o_adj[2][2] = {{0, 0}, {0, 0}};
  // PML grids: the face fields psi_x, psi_y of the forward and adjoint ping-pong
  // sets and of every checkpoint (float32), and the slots per CTA
  int pml = 0, slot_cap = 0;
  size_t o_psi[2][2] = {{0, 0}, {0, 0}};
  size_t o_apsi[2][2] = {{0, 0}, {0, 0}};
  size_t o_ckpsi = 0;
  size_t o_ckpt = 0, ckpt_elem_bytes = 4, o_scales = 0, o_seg = 0, o_graw = 0;
  size_t o_sched = 0;  // one item counter per temporally blocked launch of a pass
  int n_sched = 0;
  size_t total = 0;
  size_t smem[4] = {0, 0, 0, 0};  // per kernel mode (MODE_FWD .. MODE_FWDQ)
  // binding
  char* ws = nullptr;
  size_t ws_bytes = 0;
  bool bound = false;
  bool have_ckpt = false;
  int sm_count = 0;
  // CUDA-graph replay of the launch sequences (captured on a private stream,
  // launched on the caller's); the key holds every pointer baked into the graph
  struct Graph {
    cudaGraphExec_t exec = nullptr;
    const void* key[4] = {nullptr, nullptr, nullptr, nullptr};
    int flag = 0;
    unsigned long long used = 0;  // last replay (least recently used is replaced)
  };
  // A few captured passes per kind, keyed by their output pointers: a caller that
  // alternates output buffers (a new traces tensor per call while the previous one
  // is still alive) replays instead of capturing every call.
  static constexpr int kGraphs = 4;
  struct GraphSet {
    Graph slot[kGraphs];
  };
  GraphSet g_fwd, g_adj;
  unsigned long long graph_tick = 0;
  cudaStream_t capture_stream = nullptr;
  void drop_graphs() {
    for (GraphSet* gs : {&g_fwd, &g_adj})
      for (Graph& g : gs->slot) {
        if (g.exec) cudaGraphExecDestroy(g.exec);
        g = Graph();
      }
  }
  ~fdtd_plan() {
    drop_graphs();
    if (capture_stream) cudaStreamDestroy(capture_stream);
  }
};

int32_t fdtd::validate_grid(const fdtd_grid& g) {
  if (g.ny < 8 || g.nx < 8) return fail(FDTD_ERR_INVALID, "grid must be at least 8 x 8");
  if (g.pitch < g.nx || g.pitch % 4 != 0) return fail(FDTD_ERR_INVALID, "pitch must be a multiple of 4 and >= nx");
  if (!(g.dx > 0) || !(g.dy > 0) || !(g.dt > 0)) return fail(FDTD_ERR_INVALID, "dx, dy and dt must be positive");
  if (!g.coef || !g.mur) return fail(FDTD_ERR_INVALID, "coef and mur must be set");
  if (g.pml && (g.pml_cells < 1 || 2 * g.pml_cells >= std::min(g.nx, g.ny)))
    return fail(FDTD_ERR_INVALID, "PML layer must be at least 1 cell and thinner than half the grid");
  return FDTD_OK;
}

int32_t fdtd::validate_plain_problem(const fdtd_problem& prob) {
  int32_t rc = validate_grid(prob.grid);
  if (rc) return rc;
  if (prob.grid.pml)
    return fail(FDTD_ERR_UNSUPPORTED, "the plain per-shot forms run grids with Mur edges; a PML grid runs in the "
                                      "fused engine or with fdtd_step_pml");
  const fdtd_grid& g = prob.grid;
  if (prob.n_shots < 1 || prob.n_steps < 1) return fail(FDTD_ERR_INVALID, "n_shots and n_steps must be positive");
  const int R = prob.rx.n;
  if (R < 1 || !prob.rx.row0 || !prob.rx.col0 || !prob.rx.w) return fail(FDTD_ERR_INVALID, "receivers missing");
  for (int r = 0; r < R; ++r) {
    // a receiver samples rows row0, row0 + 1 and columns col0, col0 + 1
    if (prob.rx.row0[r] < 0 || prob.rx.row0[r] > g.ny - 2 || prob.rx.col0[r] < 0 || prob.rx.col0[r] > g.nx - 2)
      return fail(FDTD_ERR_INVALID, "receiver " + std::to_string(r) + " lies outside the grid");
  }
  const fdtd_sources& src = prob.src;
  if (src.per_shot < 0) return fail(FDTD_ERR_INVALID, "sources per shot must not be negative");
  if (src.per_shot == 0) return FDTD_OK;
  if (!src.row || !src.col || !src.w || !src.wave || !src.waveforms)
    return fail(FDTD_ERR_INVALID, "source arrays missing");
  if (src.n_waves < 1 || src.waveform_len < 0) return fail(FDTD_ERR_INVALID, "bad waveform table shape");
  const size_t n = (size_t)prob.n_shots * src.per_shot;
  for (size_t e = 0; e < n; ++e) {
    if (src.wave[e] < 0) continue;  // unused entry
    if (src.wave[e] >= src.n_waves)
      return fail(FDTD_ERR_INVALID, "source entry " + std::to_string(e) + ": waveform index out of range");
    if (src.row[e] < 0 || src.row[e] >= g.ny || src.col[e] < 0 || src.col[e] >= g.nx)
      return fail(FDTD_ERR_INVALID, "source entry " + std::to_string(e) + " lies outside the grid");
  }
  return FDTD_OK;
}

namespace {

void fill_params(const fdtd_plan* p, TbParams& q) {
  std::memset(&q, 0, sizeof(q));
  const fdtd_grid& g = p->prob.grid;
  q.ny = g.ny;
  q.nx = g.nx;
  q.pitch = g.pitch;
  const double idx2 = 1.0 / (g.dx * g.dx), idy2 = 1.0 / (g.dy * g.dy);
  q.idx2 = (float)idx2;
  q.idy2 = (float)idy2;
  q.cdiag = (float)(-2.0 * (idx2 + idy2));
  q.ratio = (float)(idx2 / idy2);
  q.qdiag = (float)(-2.0 * (1.0 + idx2 / idy2));
  q.coef = g.coef;
  q.mur = g.mur;
  q.tiles = reinterpret_cast<const TbTile*>(p->ws + p->o_tiles);
  q.ntiles = (int)p->tiles.size();
  q.nshots = p->prob.n_shots;
  q.nwarps = p->nw;
  q.taps = reinterpret_cast<const TbTap*>(p->ws + p->o_taps);
  q.tmask = reinterpret_cast<const TbMask*>(p->ws + p->o_tmask);
  q.rxl = reinterpret_cast<const int*>(p->ws + p->o_rxl);
  q.recs = reinterpret_cast<const TbRec*>(p->ws + p->o_recs);
  q.nrow_max = p->nrow_max;
  q.adj_coef = p->adj_coef;
  q.pair_sync = p->pair_sync;
  q.nrxl_max = p->nrxl_max;
  q.tmax = p->tmax;
  q.src = reinterpret_cast<const SrcNode*>(p->ws + p->o_src);
  q.nsrc_max = p->nsrc_max;
  q.stap = reinterpret_cast<const SrcTap*>(p->ws + p->o_stap);
  q.stap_off = reinterpret_cast<const int*>(p->ws + p->o_stap_off);
  q.nsrow_max = p->nsrow_max;
  q.waveforms = p->prob.src.waveforms;
  q.wave_len = p->prob.src.waveform_len;
  q.nrx = p->prob.rx.n;
  q.nt = p->prob.n_steps;
  q.seg_stride = (long long)p->field_elems;
  if (p->pml) {
    q.pml = g.pml;
    q.slot_cap = p->slot_cap;
  }
}

int grid_size(const fdtd_plan* p) {
  const int items = (int)p->tiles.size() * p->prob.n_shots;
  const int per_sm = p->tun.ctas_per_sm > 0 ? p->tun.ctas_per_sm : 1;
  const int g = p->sm_count * per_sm;
  return std::max(1, std::min(items, g));
}

float* fptr(fdtd_plan* p, size_t off) { return reinterpret_cast<float*>(p->ws + off); }

int32_t launch(fdtd_plan* p, TbParams& q, int mode, cudaStream_t st) {
  // 85 % of the items in static runs of consecutive shots, the rest dealt out one
  // by one to whichever CTA is free (the tail balances; the runs reuse tiles). A
  // PML grid's layer tiles cost several times an interior tile, more than the
  // dealt-out rest could balance: there every item is dealt out, costliest first.
  const int grid = grid_size(p);
  const int items = (int)p->tiles.size() * p->prob.n_shots;
  q.static_items = (q.sched && mode == MODE_FWD && !p->pml) ? (int)(0.85 * items / grid) : 0;
  cudaError_t e = tb_launch(q, p->ky, mode, grid, p->smem[mode], st);
  if (e != cudaSuccess) return cuda_fail(e, "temporally blocked kernel launch");
  return FDTD_OK;
}

int32_t build_tables(fdtd_plan* p, const fdtd_problem* prob) {
  const fdtd_grid& g = prob->grid;
  const int ny = g.ny, nx = g.nx, KY = p->ky, RY = p->RY;
  const int halo = p->tmax + 1;
  // gradient plans: the x halo rounded up to whole lanes (4 columns), so that every
  // interior ownership boundary falls between lanes and the recompute stores its
  // Laplacian stream as whole 16-byte rows
  const int halo_x = p->for_gradient ? (halo + 3) / 4 * 4 : halo;
  p->pml = g.pml ? g.pml_cells : 0;
  p->slot_cap = 0;
  std::vector<AxisTile> tx, ty;
  std::string err = tile_axis(nx, RX, 4, halo_x, 0, tx);
  if (!err.empty()) return fail(FDTD_ERR_UNSUPPORTED, "x tiling: " + err);
  err = tile_axis(ny, RY, 1, halo, KY, ty);
  if (!err.empty()) return fail(FDTD_ERR_UNSUPPORTED, "y tiling: " + err);

  // receivers -> unique tap nodes, contributions in the reference's
  // index_put_ order (all w00 taps, then w10, w01, w11)
  const int R = prob->rx.n;
  std::map<std::pair<int, int>, int> node_id;
  std::vector<std::pair<int, int>> nodes;
  std::vector<std::vector<std::pair<int, float>>> contrib;
  for (int tap = 0; tap < 4; ++tap) {
    for (int r = 0; r < R; ++r) {
      const int r0 = prob->rx.row0[r], c0 = prob->rx.col0[r];
      const int row = r0 + (tap >= 2 ? 1 : 0), col = c0 + (tap & 1);
      auto key = std::make_pair(row, col);
      auto it = node_id.find(key);
      int id;
      if (it == node_id.end()) {
        id = (int)nodes.size();
        node_id[key] = id;
        nodes.push_back(key);
        contrib.emplace_back();
      } else {
        id = it->second;
      }
      contrib[id].push_back({r, prob->rx.w[4 * r + tap]});
      if ((int)contrib[id].size() > TAP_C) return fail(FDTD_ERR_UNSUPPORTED, "more than 8 receiver taps share one grid node");
    }
  }
  for (int r = 0; r < R; ++r) {
    const int r0 = prob->rx.row0[r], c0 = prob->rx.col0[r];
    if (r0 < 0 || r0 > ny - 2 || c0 < 0 || c0 > nx - 2)
      return fail(FDTD_ERR_INVALID, "receiver " + std::to_string(r) + " lies outside the grid");
  }

  p->tiles.clear();
  p->taps.clear();
  p->tmask.clear();
  p->rxl.clear();
  p->recs.clear();
  p->nrow_max = 0;
  p->nrxl_max = 0;
  std::vector<int> recorded(R, 0);
  // Tiles in decreasing order of cost (Mur edges and corners first, then tiles
  // with receiver taps, interior tiles last). Items are (tile, shot) pairs dealt
  // out to the persistent CTAs with a grid stride in this order, so the partial
  // last round of a launch holds the cheapest items.
  struct Order { int cost, j, i; };  // indices into ty, tx
  std::vector<Order> order;
  for (size_t j = 0; j < ty.size(); ++j)
    for (size_t i = 0; i < tx.size(); ++i) {
      const int fy = ty[j].flags, fx = tx[i].flags;
      const int edges = ((fy & 1) != 0) + ((fy & 2) != 0) + ((fx & 1) != 0) + ((fx & 2) != 0);
      bool taps = false;
      for (const auto& nd : nodes) {
        const int ly = nd.first - ty[j].origin, lx = nd.second - tx[i].origin;
        if (ly >= 0 && ly < RY && lx >= 0 && lx < RX) { taps = true; break; }
      }
      order.push_back({2 * edges + (taps ? 1 : 0), (int)j, (int)i});
    }
  std::stable_sort(order.begin(), order.end(), [](const Order& a, const Order& b) { return a.cost > b.cost; });
  for (const Order& o : order) {
    {
      const AxisTile& ay = ty[o.j];
      const AxisTile& ax = tx[o.i];
      TbTile t;
      std::memset(&t, 0, sizeof(t));
      t.rx0 = ax.origin;
      t.ry0 = ay.origin;
      t.ox0 = ax.own0;
      t.ox1 = ax.own1;
      t.oy0 = ay.own0;
      t.oy1 = ay.own1;
      t.flags = ((ax.flags & 1) ? TF_LEFT : 0) | ((ax.flags & 2) ? TF_RIGHT : 0) |
                ((ay.flags & 1) ? TF_BOTTOM : 0) | ((ay.flags & 2) ? TF_TOP : 0) |
                (((ax.flags | ay.flags) & 4) ? TF_OUTSIDE : 0);
      if ((t.flags & TF_LEFT) && t.rx0 != 0) return fail(FDTD_ERR_UNSUPPORTED, "left edge tile must start at column 0");
      if (g.pml) {
        // no Mur edges; a region holding layer cells is a PML tile, and each of its
        // threads whose columns or rows enter the layer takes a slot
        t.flags &= ~TF_MUR;
        const int P = g.pml_cells;
        auto in_layer = [](int v, int n, int P) { return v >= 0 && v < n && (v < P || v >= n - P); };
        int slots = 0;
        for (int w = 0; w < p->nw; ++w) {
          bool rows = false;
          for (int r = 0; r < KY; ++r) rows = rows || in_layer(t.ry0 + w * KY + r, ny, P);
          for (int l = 0; l < 32; ++l) {
            bool cols = false;
            for (int c = 0; c < 4; ++c) cols = cols || in_layer(t.rx0 + 4 * l + c, nx, P);
            if (rows || cols) ++slots;
          }
        }
        if (slots > 0) t.flags |= TF_PML;
        p->slot_cap = std::max(p->slot_cap, slots);
      }
      // taps inside the region, sorted by (thread, bit)
      std::vector<std::pair<int, int>> local;  // (packed, node id)
      for (size_t id = 0; id < nodes.size(); ++id) {
        const int ly = nodes[id].first - t.ry0, lx = nodes[id].second - t.rx0;
        if (ly < 0 || ly >= RY || lx < 0 || lx >= RX) continue;
        const int packed = (((ly / KY) * 32 + (lx >> 2)) << 8) | ((ly % KY) * 4 + (lx & 3));
        local.push_back({packed, (int)id});
      }
      std::sort(local.begin(), local.end());
      std::map<int, int> rloc;
      std::vector<int> rx_here;
      for (auto& pr : local)
        for (auto& cw : contrib[pr.second])
          if (!rloc.count(cw.first)) { rloc[cw.first] = 0; }
      for (auto& kv : rloc) { kv.second = (int)rx_here.size(); rx_here.push_back(kv.first); }
      t.tap_off = (int)p->taps.size();
      t.ntap = (int)local.size();
      const size_t mbase = p->tmask.size();
      p->tmask.resize(mbase + (size_t)p->nw * 32, TbMask{0u, 0x7fffffff});
      std::map<int, int> slot_of_node;  // node id -> staged float (srow * 4 + column)
      t.nrow = 0;
      for (size_t i = 0; i < local.size(); ++i) {
        TbTap tp;
        tp.packed = local[i].first;
        // taps are sorted by (thread, row, column): a new (thread, row) pair opens a staged row
        if (i == 0 || (local[i].first >> 2) != (local[i - 1].first >> 2)) ++t.nrow;
        tp.srow = t.nrow - 1;
        for (int q = 0; q < TAP_C; ++q) { tp.rloc[q] = -1; tp.w[q] = 0.f; }
        const auto& cl = contrib[local[i].second];
        for (size_t q = 0; q < cl.size(); ++q) {
          tp.rloc[q] = rloc[cl[q].first];
          tp.w[q] = cl[q].second;
        }
        p->taps.push_back(tp);
        TbMask& mk = p->tmask[mbase + (tp.packed >> 8)];
        mk.mask |= 1u << ((tp.packed & 255) >> 2);
        mk.base = std::min(mk.base, tp.srow);
        slot_of_node[local[i].second] = tp.srow * 4 + (tp.packed & 3);
      }
      t.rxl_off = (int)p->rxl.size();
      t.nrxl = (int)rx_here.size();
      p->rxl.insert(p->rxl.end(), rx_here.begin(), rx_here.end());
      t.rec_off = (int)p->recs.size();
      for (int r = 0; r < R; ++r) {
        const int r0 = prob->rx.row0[r], c0 = prob->rx.col0[r];
        if (r0 < t.oy0 || r0 >= t.oy1 || c0 < t.ox0 || c0 >= t.ox1) continue;
        TbRec rc;
        rc.rg = r;
        for (int tap = 0; tap < 4; ++tap) {
          const int id = node_id[{r0 + (tap >= 2 ? 1 : 0), c0 + (tap & 1)}];
          auto it = slot_of_node.find(id);
          if (it == slot_of_node.end()) return fail(FDTD_ERR_UNSUPPORTED, "receiver footprint outside its tile");
          rc.slot[tap] = it->second;
          rc.w[tap] = prob->rx.w[4 * r + tap];
        }
        p->recs.push_back(rc);
        recorded[r]++;
      }
      t.nrec = (int)p->recs.size() - t.rec_off;
      p->nrow_max = std::max(p->nrow_max, t.nrow);
      p->nrxl_max = std::max(p->nrxl_max, t.nrxl);
      p->tiles.push_back(t);
    }
  }
  for (int r = 0; r < R; ++r)
    if (recorded[r] != 1) return fail(FDTD_ERR_UNSUPPORTED, "receiver not recorded exactly once");

  // per-shot injection nodes, duplicates merged in entry order
  const int S = prob->n_shots, K = prob->src.per_shot;
  std::vector<std::vector<SrcNode>> shot_nodes(S);
  for (int s = 0; s < S; ++s) {
    std::map<std::pair<int, int>, int> where;
    auto& list = shot_nodes[s];
    for (int j = 0; j < K; ++j) {
      const int e = s * K + j;
      if (prob->src.wave[e] < 0) continue;
      const int row = prob->src.row[e], col = prob->src.col[e];
      if (row < 0 || row >= ny || col < 0 || col >= nx) return fail(FDTD_ERR_INVALID, "source outside the grid");
      if (prob->src.wave[e] >= prob->src.n_waves) return fail(FDTD_ERR_INVALID, "source waveform index out of range");
      auto it = where.find({row, col});
      int found;
      if (it == where.end()) {
        SrcNode sn;
        sn.row = row;
        sn.col = col;
        for (int q = 0; q < SRC_C; ++q) { sn.wave[q] = -1; sn.w[q] = 0.f; }
        found = (int)list.size();
        where[{row, col}] = found;
        list.push_back(sn);
      } else {
        found = it->second;
      }
      SrcNode& sn = list[found];
      int q = 0;
      while (q < SRC_C && sn.wave[q] >= 0) ++q;
      if (q == SRC_C) return fail(FDTD_ERR_UNSUPPORTED, "more than 4 source entries on one node");
      sn.wave[q] = prob->src.wave[e];
      sn.w[q] = prob->src.w[e];
    }
  }
  p->nsrc_max = 1;
  for (int s = 0; s < S; ++s) p->nsrc_max = std::max(p->nsrc_max, (int)shot_nodes[s].size());
  p->src.assign((size_t)S * p->nsrc_max, SrcNode());
  p->nsrc.assign(S, 0);
  for (int s = 0; s < S; ++s) {
    p->nsrc[s] = (int)shot_nodes[s].size();
    std::copy(shot_nodes[s].begin(), shot_nodes[s].end(), p->src.begin() + (size_t)s * p->nsrc_max);
  }
  // per (shot, tile): the nodes inside the region, sorted by (thread, row, column);
  // every (thread, band row) holding one is a staged source row
  const int NT = (int)p->tiles.size();
  p->stap.clear();
  p->stap_off.assign((size_t)S * NT + 1, 0);
  p->nsrow_max = 0;
  for (int s = 0; s < S; ++s) {
    for (int ti = 0; ti < NT; ++ti) {
      const TbTile& t = p->tiles[ti];
      p->stap_off[(size_t)s * NT + ti] = (int)p->stap.size();
      std::vector<std::pair<int, int>> local;  // (packed, node)
      for (int j = 0; j < p->nsrc[s]; ++j) {
        const SrcNode& sn = shot_nodes[s][j];
        const int ly = sn.row - t.ry0, lx = sn.col - t.rx0;
        if (ly < 0 || ly >= RY || lx < 0 || lx >= RX) continue;
        local.push_back({(((ly / KY) * 32 + (lx >> 2)) << 8) | ((ly % KY) * 4 + (lx & 3)), j});
      }
      std::sort(local.begin(), local.end());
      int nrow = 0;
      for (size_t i = 0; i < local.size(); ++i) {
        if (i == 0 || (local[i].first >> 2) != (local[i - 1].first >> 2)) ++nrow;
        SrcTap st;
        st.packed = local[i].first;
        st.srow = nrow - 1;
        st.node = local[i].second;
        st.pad = 0;
        p->stap.push_back(st);
      }
      p->nsrow_max = std::max(p->nsrow_max, nrow);
    }
  }
  p->stap_off[(size_t)S * NT] = (int)p->stap.size();
  return FDTD_OK;
}

}  // namespace

extern "C" {

int32_t fdtd_abi_version(void) { return FDTD_ABI_VERSION; }

const char* fdtd_last_error(void) { return g_error.c_str(); }

int32_t fdtd_tile_axis(int32_t n, int32_t region, int32_t align, int32_t halo, int32_t band,
                       int32_t max_tiles, int32_t* out, int32_t* n_tiles) {
  std::vector<AxisTile> t;
  std::string err = tile_axis(n, region, align, halo, band, t);
  if (!err.empty()) return fail(FDTD_ERR_UNSUPPORTED, err);
  if (n_tiles) *n_tiles = (int32_t)t.size();
  if ((int)t.size() > max_tiles) return fail(FDTD_ERR_INVALID, "output too small");
  for (size_t i = 0; i < t.size(); ++i) {
    out[4 * i] = t[i].origin;
    out[4 * i + 1] = t[i].own0;
    out[4 * i + 2] = t[i].own1;
    out[4 * i + 3] = t[i].flags;
  }
  return FDTD_OK;
}

int32_t fdtd_tap_table(int32_t ny, int32_t nx, const fdtd_receivers* rx, int32_t* tap_nodes,
                       float* tap_w, int32_t* n_nodes) {
  if (!rx || !n_nodes) return fail(FDTD_ERR_INVALID, "null argument");
  std::map<std::pair<int, int>, int> node_id;
  std::vector<std::pair<int, int>> nodes;
  std::vector<std::vector<std::pair<int, float>>> contrib;
  for (int tap = 0; tap < 4; ++tap) {
    for (int r = 0; r < rx->n; ++r) {
      const int row = rx->row0[r] + (tap >= 2 ? 1 : 0), col = rx->col0[r] + (tap & 1);
      if (row < 0 || row >= ny || col < 0 || col >= nx) return fail(FDTD_ERR_INVALID, "receiver outside the grid");
      auto key = std::make_pair(row, col);
      auto it = node_id.find(key);
      int id;
      if (it == node_id.end()) {
        id = (int)nodes.size();
        node_id[key] = id;
        nodes.push_back(key);
        contrib.emplace_back();
      } else {
        id = it->second;
      }
      contrib[id].push_back({r, rx->w[4 * r + tap]});
      if ((int)contrib[id].size() > TAP_C) return fail(FDTD_ERR_UNSUPPORTED, "more than 8 receiver taps share one grid node");
    }
  }
  const int cap = *n_nodes;
  *n_nodes = (int32_t)nodes.size();
  if ((int)nodes.size() > cap) return fail(FDTD_ERR_INVALID, "tap table capacity too small");
  for (size_t i = 0; i < nodes.size(); ++i) {
    int32_t* nd = tap_nodes + i * (2 + TAP_C);
    nd[0] = nodes[i].first;
    nd[1] = nodes[i].second;
    for (int q = 0; q < TAP_C; ++q) {
      const bool used = q < (int)contrib[i].size();
      nd[2 + q] = used ? contrib[i][q].first : -1;
      tap_w[i * TAP_C + q] = used ? contrib[i][q].second : 0.f;
    }
  }
  return FDTD_OK;
}

int32_t fdtd_prepare_medium(const double* c, int32_t ny, int32_t nx, int32_t pitch, double dt,
                            double dx, double dy, float* coef, float* mur, void* stream) {
  if (!c || !coef || !mur) return fail(FDTD_ERR_INVALID, "null pointer");
  if (ny < 3 || nx < 3 || pitch < nx || pitch % 4) return fail(FDTD_ERR_INVALID, "bad grid shape");
  if (!(dt > 0) || !(dx > 0) || !(dy > 0)) return fail(FDTD_ERR_INVALID, "dt, dx and dy must be positive");
  cudaError_t e = prepare_medium_launch(c, ny, nx, pitch, dt, dx, dy, coef, mur, (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(e, "prepare_medium");
  return FDTD_OK;
}

int32_t fdtd_prepare_medium_pml(const double* c, int32_t ny, int32_t nx, int32_t pitch, double dt, double dx,
                                double dy, int32_t cells, double reflection, float* coef, float* mur, float* pml,
                                void* stream) {
  if (!c || !coef || !mur || !pml) return fail(FDTD_ERR_INVALID, "null pointer");
  if (ny < 8 || nx < 8 || pitch < nx || pitch % 4) return fail(FDTD_ERR_INVALID, "bad grid shape");
  if (!(dt > 0) || !(dx > 0) || !(dy > 0)) return fail(FDTD_ERR_INVALID, "dx, dy and dt must be positive");
  if (cells < 1 || 2 * cells >= std::min(nx, ny)) return fail(FDTD_ERR_INVALID, "bad PML thickness");
  if (!(reflection > 0 && reflection < 1)) return fail(FDTD_ERR_INVALID, "reflection must lie in (0, 1)");
  cudaError_t e = prepare_medium_launch(c, ny, nx, pitch, dt, dx, dy, coef, mur, (cudaStream_t)stream);
  if (e == cudaSuccess)
    e = prepare_pml_launch(c, ny, nx, pitch, dt, dx, dy, cells, reflection, coef, pml, (cudaStream_t)stream);
  return e == cudaSuccess ? FDTD_OK : cuda_fail(e, "prepare_medium_pml");
}

int32_t fdtd_step_pml(const fdtd_grid* grid, int32_t n_shots, const float* u_old, const float* u, float* u_next,
                      const float* psx, const float* psy, float* psx_next, float* psy_next, int32_t src_per_shot,
                      const int32_t* src_row, const int32_t* src_col, const float* src_w, const int32_t* src_wave,
                      const float* waveforms, int32_t waveform_len, int32_t step, const float* dense,
                      int32_t adjoint, void* stream) {
  if (!grid) return fail(FDTD_ERR_INVALID, "null grid");
  int32_t rc = validate_grid(*grid);
  if (rc) return rc;
  if (!grid->pml) return fail(FDTD_ERR_INVALID, "fdtd_step_pml needs a grid with PML tables");
  if (n_shots < 1 || !u_old || !u || !u_next || !psx || !psy || !psx_next || !psy_next)
    return fail(FDTD_ERR_INVALID, "null field");
  if (adjoint != 0 && adjoint != 2) return fail(FDTD_ERR_INVALID, "adjoint must be 0 or 2 on a PML grid");
  if (src_per_shot > 0 && (!src_row || !src_col || !src_w || !src_wave || !waveforms))
    return fail(FDTD_ERR_INVALID, "source arrays missing");
  StepArgs a;
  a.ny = grid->ny;
  a.nx = grid->nx;
  a.pitch = grid->pitch;
  const double idx2 = 1.0 / (grid->dx * grid->dx), idy2 = 1.0 / (grid->dy * grid->dy);
  a.idx2 = (float)idx2;
  a.idy2 = (float)idy2;
  a.cdiag = (float)(-2.0 * (idx2 + idy2));
  a.ratio = (float)(idx2 / idy2);
  a.qdiag = (float)(-2.0 * (1.0 + idx2 / idy2));
  a.coef = grid->coef;
  a.mur = grid->mur;
  a.n_shots = n_shots;
  a.u_old = u_old;
  a.u = u;
  a.u_next = u_next;
  a.src_per_shot = src_per_shot > 0 ? src_per_shot : 0;
  a.src_row = src_row;
  a.src_col = src_col;
  a.src_w = src_w;
  a.src_wave = src_wave;
  a.waveforms = waveforms;
  a.wave_len = waveform_len;
  a.step = step;
  a.dense = dense;
  a.adjoint = adjoint;
  cudaError_t e = step_pml_launch(a, grid->pml, psx, psy,
                                  psx_next, psy_next, (cudaStream_t)stream);
  return e == cudaSuccess ? FDTD_OK : cuda_fail(e, "fdtd_step_pml");
}

}  // extern "C"

namespace {

// One step of the one-step kernel for the Mur grid, or with `density` the
// variable-density operator (adjoint 0 or 1).
int32_t step_impl(const fdtd_grid* grid, const fdtd_density* density, int32_t n_shots, const float* u_old,
                  const float* u, float* u_next, int32_t src_per_shot, const int32_t* src_row,
                  const int32_t* src_col, const float* src_w, const int32_t* src_wave,
                  const float* waveforms, int32_t waveform_len, int32_t step, const float* dense,
                  int32_t adjoint, void* stream) {
  if (!grid) return fail(FDTD_ERR_INVALID, "null grid");
  if (grid->ny < 3 || grid->nx < 3 || grid->pitch < grid->nx || grid->pitch % 4)
    return fail(FDTD_ERR_INVALID, "bad grid shape");
  if (!grid->coef || !grid->mur || !u_old || !u || !u_next) return fail(FDTD_ERR_INVALID, "null pointer");
  if (grid->pml) return fail(FDTD_ERR_INVALID, "a PML grid steps with fdtd_step_pml");
  if (u_next == u || u_next == u_old) return fail(FDTD_ERR_INVALID, "u_next must not alias the inputs");
  if (n_shots < 1) return fail(FDTD_ERR_INVALID, "n_shots must be positive");
  if (src_per_shot > 0 && (!src_row || !src_col || !src_w || !src_wave || !waveforms))
    return fail(FDTD_ERR_INVALID, "source arrays missing");
  StepArgs a;
  a.ny = grid->ny;
  a.nx = grid->nx;
  a.pitch = grid->pitch;
  const double idx2 = 1.0 / (grid->dx * grid->dx), idy2 = 1.0 / (grid->dy * grid->dy);
  a.idx2 = (float)idx2;
  a.idy2 = (float)idy2;
  a.cdiag = (float)(-2.0 * (idx2 + idy2));
  a.ratio = (float)(idx2 / idy2);
  a.qdiag = (float)(-2.0 * (1.0 + idx2 / idy2));
  a.coef = grid->coef;
  a.mur = grid->mur;
  a.n_shots = n_shots;
  a.u_old = u_old;
  a.u = u;
  a.u_next = u_next;
  a.src_per_shot = src_per_shot > 0 ? src_per_shot : 0;
  a.src_row = src_row;
  a.src_col = src_col;
  a.src_w = src_w;
  a.src_wave = src_wave;
  a.waveforms = waveforms;
  a.wave_len = waveform_len;
  a.step = step;
  a.dense = dense;
  if (adjoint < 0 || adjoint > 2) return fail(FDTD_ERR_INVALID, "adjoint must be 0, 1 or 2");
  a.adjoint = adjoint;
  if (density) {
    if (!density->kappa || !density->bx || !density->by) return fail(FDTD_ERR_INVALID, "density arrays missing");
    if (adjoint == 2) return fail(FDTD_ERR_INVALID, "a variable-density step takes adjoint 0 or 1");
    a.kap = density->kappa;
    a.bx = density->bx;
    a.by = density->by;
  }
  cudaError_t e = step_launch(a, (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(e, "step");
  return FDTD_OK;
}

}  // namespace

extern "C" {

int32_t fdtd_step(const fdtd_grid* grid, int32_t n_shots, const float* u_old, const float* u,
                  float* u_next, int32_t src_per_shot, const int32_t* src_row,
                  const int32_t* src_col, const float* src_w, const int32_t* src_wave,
                  const float* waveforms, int32_t waveform_len, int32_t step, const float* dense,
                  int32_t adjoint, void* stream) {
  return step_impl(grid, nullptr, n_shots, u_old, u, u_next, src_per_shot, src_row, src_col, src_w, src_wave,
                   waveforms, waveform_len, step, dense, adjoint, stream);
}

int32_t fdtd_step_density(const fdtd_grid* grid, const fdtd_density* density, int32_t n_shots, const float* u_old,
                          const float* u, float* u_next, int32_t src_per_shot, const int32_t* src_row,
                          const int32_t* src_col, const float* src_w, const int32_t* src_wave,
                          const float* waveforms, int32_t waveform_len, int32_t step, const float* dense,
                          int32_t adjoint, void* stream) {
  if (!density) return fail(FDTD_ERR_INVALID, "null density");
  return step_impl(grid, density, n_shots, u_old, u, u_next, src_per_shot, src_row, src_col, src_w, src_wave,
                   waveforms, waveform_len, step, dense, adjoint, stream);
}

int32_t fdtd_prepare_density(const double* c, const double* rho, int32_t ny, int32_t nx, int32_t pitch, double dt,
                             double dx, double dy, float* kappa, float* bx, float* by, float* mur, void* stream) {
  if (!c || !rho || !kappa || !bx || !by || !mur) return fail(FDTD_ERR_INVALID, "null pointer");
  if (ny < 3 || nx < 3 || pitch < nx || pitch % 4) return fail(FDTD_ERR_INVALID, "bad grid shape");
  if (!(dt > 0) || !(dx > 0) || !(dy > 0)) return fail(FDTD_ERR_INVALID, "dx, dy and dt must be positive");
  cudaError_t e = prepare_density_launch(c, rho, ny, nx, pitch, dt, dx, dy, kappa, bx, by, mur, (cudaStream_t)stream);
  return e == cudaSuccess ? FDTD_OK : cuda_fail(e, "prepare_density");
}

int32_t fdtd_density_chain_rule(int32_t ny, int32_t nx, int32_t pitch, const double* m, const double* rho,
                                const double* g_kappa, const double* g_bx, const double* g_by, const uint8_t* mask,
                                double* g_m, double* g_rho, void* stream) {
  if (!m || !rho || !g_kappa || !g_bx || !g_by || !g_m || !g_rho) return fail(FDTD_ERR_INVALID, "null pointer");
  if (ny < 3 || nx < 3 || pitch < nx) return fail(FDTD_ERR_INVALID, "bad grid shape");
  cudaError_t e = density_chain_launch(ny, nx, pitch, m, rho, g_kappa, g_bx, g_by, mask, g_m, g_rho,
                                       (cudaStream_t)stream);
  return e == cudaSuccess ? FDTD_OK : cuda_fail(e, "density_chain_rule");
}

int32_t fdtd_gather(const fdtd_grid* grid, int32_t n_shots, const float* fields, int32_t n_rx,
                    const int32_t* rx_rc, const float* rx_w, float* out, int64_t out_shot_stride,
                    int64_t out_rx_stride, void* stream) {
  if (!grid || !fields || !rx_rc || !rx_w || !out) return fail(FDTD_ERR_INVALID, "null pointer");
  if (n_shots < 1 || n_rx < 0) return fail(FDTD_ERR_INVALID, "bad sizes");
  if (n_rx == 0) return FDTD_OK;
  cudaError_t e = gather_launch(grid->ny, grid->pitch, n_shots, fields, n_rx, rx_rc, rx_w, out,
                                out_shot_stride, out_rx_stride, (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(e, "gather");
  return FDTD_OK;
}

int32_t fdtd_scatter(const fdtd_grid* grid, int32_t n_shots, int32_t n_nodes,
                     const int32_t* tap_nodes, const float* tap_w, const float* residual,
                     int64_t res_shot_stride, int64_t res_rx_stride, float* dense, void* stream) {
  if (!grid || !tap_nodes || !tap_w || !residual || !dense) return fail(FDTD_ERR_INVALID, "null pointer");
  if (n_shots < 1 || n_nodes < 0) return fail(FDTD_ERR_INVALID, "bad sizes");
  if (n_nodes == 0) return FDTD_OK;
  cudaError_t e = scatter_launch(grid->ny, grid->pitch, n_shots, n_nodes, tap_nodes, tap_w, residual,
                                 res_shot_stride, res_rx_stride, dense, (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(e, "scatter");
  return FDTD_OK;
}

int32_t fdtd_image(const fdtd_grid* grid, int32_t n_shots, const float* adj, const float* fwd,
                   double scale, double* g, void* stream) {
  if (!grid || !adj || !fwd || !g) return fail(FDTD_ERR_INVALID, "null pointer");
  const double idx2 = 1.0 / (grid->dx * grid->dx), idy2 = 1.0 / (grid->dy * grid->dy);
  cudaError_t e = image_launch(grid->ny, grid->nx, grid->pitch, (float)idx2, (float)idy2,
                               (float)(-2.0 * (idx2 + idy2)), n_shots, adj, fwd, scale, nullptr, g,
                               (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(e, "image");
  return FDTD_OK;
}

int32_t fdtd_residual_misfit(int32_t n_shots, int32_t n_rx, int32_t n_steps, const float* traces,
                             const float* observed, int64_t observed_shot_stride,
                             const int32_t* mute, float* residual, double* misfit, void* stream) {
  if (!traces || !observed || !residual || !misfit) return fail(FDTD_ERR_INVALID, "null pointer");
  if (n_shots < 1 || n_rx < 1 || n_steps < 1) return fail(FDTD_ERR_INVALID, "bad sizes");
  cudaError_t e = residual_launch(n_shots, n_rx, n_steps, traces, observed, observed_shot_stride,
                                  mute, residual, misfit, (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(e, "residual");
  return FDTD_OK;
}

int32_t fdtd_chain_rule(int64_t n, const double* grad_c2, const double* m, const uint8_t* mask,
                        double* g_m, void* stream) {
  if (!grad_c2 || !m || !g_m) return fail(FDTD_ERR_INVALID, "null pointer");
  if (n < 0) return fail(FDTD_ERR_INVALID, "bad size");
  if (n == 0) return FDTD_OK;
  cudaError_t e = chain_rule_launch(n, grad_c2, m, mask, g_m, (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(e, "chain rule");
  return FDTD_OK;
}

// ----------------------------------------------------------------- plans

int32_t fdtd_plan_create(const fdtd_problem* problem, const fdtd_tuning* tuning,
                         int32_t for_gradient, fdtd_plan** out) {
  if (!problem || !out) return fail(FDTD_ERR_INVALID, "null argument");
  *out = nullptr;
  int32_t rc = validate_grid(problem->grid);
  if (rc) return rc;
  if (problem->n_shots < 1 || problem->n_steps < 1) return fail(FDTD_ERR_INVALID, "n_shots and n_steps must be positive");
  if (problem->rx.n < 1 || !problem->rx.row0 || !problem->rx.col0 || !problem->rx.w)
    return fail(FDTD_ERR_INVALID, "receivers missing");
  if (problem->src.per_shot < 0 || (problem->src.per_shot > 0 &&
      (!problem->src.row || !problem->src.col || !problem->src.w || !problem->src.wave || !problem->src.waveforms)))
    return fail(FDTD_ERR_INVALID, "source arrays missing");
  fdtd_plan* p = new fdtd_plan();
  p->prob = *problem;
  fdtd_tuning t;
  std::memset(&t, 0, sizeof(t));
  if (tuning) t = *tuning;
  if (t.rows_per_lane == 0) t.rows_per_lane = 8;
  if (t.rows_per_lane != 4 && t.rows_per_lane != 8) { delete p; return fail(FDTD_ERR_UNSUPPORTED, "rows_per_lane must be 4 or 8"); }
  const int max_warps = t.rows_per_lane == 4 ? 32 : 16;
  if (t.warps == 0) t.warps = 16;
  if (t.warps < 2 || t.warps > max_warps) { delete p; return fail(FDTD_ERR_UNSUPPORTED, "warps out of range"); }
  if (t.steps_per_launch == 0) {
    // Fewest computed cells per useful cell-update: tiles(T) * (T + 3) / T, where
    // the 3 stands for the per-item load / setup / store cost in steps.
    double best = 1e300;
    int best_t = 8;
    const int ry = t.rows_per_lane * t.warps;
    for (int T = 4; T <= 32; ++T) {
      std::vector<AxisTile> ax, ay;
      if (!tile_axis(problem->grid.nx, RX, 4, T + 1, 0, ax).empty()) continue;
      if (!tile_axis(problem->grid.ny, ry, 1, T + 1, t.rows_per_lane, ay).empty()) continue;
      const int Teff = std::min(T, problem->n_steps);
      const double cost = (double)ax.size() * ay.size() * (Teff + 3.0) / Teff;
      if (cost <= best * (1.0 + 1e-9)) { best = cost; best_t = T; }
      if (T >= problem->n_steps) break;
    }
    t.steps_per_launch = best_t;
  }
  if (t.steps_per_launch < 1 || t.steps_per_launch > 48) { delete p; return fail(FDTD_ERR_UNSUPPORTED, "steps_per_launch must be in [1, 48]"); }
  if (t.ctas_per_sm == 0) t.ctas_per_sm = 1;
  if (t.step_sync < FDTD_SYNC_AUTO || t.step_sync > FDTD_SYNC_PAIR) { delete p; return fail(FDTD_ERR_INVALID, "bad step_sync"); }
  if (t.step_sync == FDTD_SYNC_PAIR && t.warps > 16) {
    delete p;
    return fail(FDTD_ERR_UNSUPPORTED, "step_sync PAIR needs at most 16 warps (15 named barriers)");
  }
  if (t.step_sync == FDTD_SYNC_AUTO) t.step_sync = t.warps <= 16 ? FDTD_SYNC_PAIR : FDTD_SYNC_CTA;
  p->pair_sync = t.step_sync == FDTD_SYNC_PAIR;
  if (t.ckpt_store < 0 || t.ckpt_store > 2) { delete p; return fail(FDTD_ERR_INVALID, "bad checkpoint storage type"); }
  p->ky = t.rows_per_lane;
  p->nw = t.warps;
  p->RY = p->ky * p->nw;
  p->tmax = t.steps_per_launch;
  p->for_gradient = for_gradient ? 1 : 0;
  const int nt = problem->n_steps;
  if (t.ckpt_every <= 0) {
    const int c = (int)std::ceil(std::sqrt(2.0 * nt));
    t.ckpt_every = ((c + p->tmax - 1) / p->tmax) * p->tmax;
  }
  // checkpoints sit on temporal-block boundaries: round the spacing up to a multiple of T
  t.ckpt_every = ((t.ckpt_every + p->tmax - 1) / p->tmax) * p->tmax;
  p->ckpt_every = t.ckpt_every;
  p->nseg = (nt + p->ckpt_every - 1) / p->ckpt_every;
  p->tun = t;
  rc = build_tables(p, problem);
  if (rc) { delete p; return rc; }
  // the adjoint keeps its coefficient tile in shared memory when that fits
  p->adj_coef = tb_smem_layout(p->nw, p->ky, MODE_ADJ, p->nrow_max, p->nrxl_max, p->tmax, 1, p->nsrow_max,
                               p->slot_cap).total <= SMEM_LIMIT;
  p->kept = 0;
  if (for_gradient && !p->pml) {
    const int want = t.kept_segments == 0 ? 1 : t.kept_segments;
    p->kept = want < 0 ? 0 : std::min(want, p->nseg);
  }
  p->tun.kept_segments = for_gradient ? (p->kept > 0 ? p->kept : -1) : t.kept_segments;
  for (int m = 0; m < 4; ++m) {
    p->smem[m] = tb_smem_layout(p->nw, p->ky, m, p->nrow_max, p->nrxl_max, p->tmax, p->adj_coef, p->nsrow_max,
                                p->slot_cap).total;
    if (p->smem[m] > SMEM_LIMIT && (m == MODE_FWD || (for_gradient && (m != MODE_FWDQ || p->kept > 0)))) {
      delete p;
      return fail(FDTD_ERR_UNSUPPORTED, "shared memory need exceeds 227 KB; use fewer steps per launch or warps");
    }
  }
  // workspace layout
  const fdtd_grid& g = problem->grid;
  p->field_elems = (size_t)problem->n_shots * g.ny * g.pitch;
  const size_t fb = p->field_elems * sizeof(float);
  size_t off = 0;
  p->o_tiles = off; off = align_up(off + p->tiles.size() * sizeof(TbTile));
  {
    // launches per pass: the forward ceil(nt / T); the adjoint pass recomputes and
    // images every segment (ceil(C / T) launches each way per segment)
    const int nt = problem->n_steps, T = p->tmax;
    const int fwd = (nt + T - 1) / T;
    const int seg = (p->ckpt_every + T - 1) / T;
    p->n_sched = std::max(fwd, p->for_gradient ? 2 * seg * p->nseg : 0) + 1;
    p->o_sched = off; off = align_up(off + (size_t)p->n_sched * sizeof(int));
  }
  p->o_taps = off; off = align_up(off + std::max<size_t>(1, p->taps.size()) * sizeof(TbTap));
  p->o_tmask = off; off = align_up(off + p->tmask.size() * sizeof(TbMask));
  p->o_rxl = off; off = align_up(off + std::max<size_t>(1, p->rxl.size()) * sizeof(int));
  p->o_recs = off; off = align_up(off + std::max<size_t>(1, p->recs.size()) * sizeof(TbRec));
  p->o_src = off; off = align_up(off + p->src.size() * sizeof(SrcNode));
  p->o_stap = off; off = align_up(off + std::max<size_t>(1, p->stap.size()) * sizeof(SrcTap));
  p->o_stap_off = off; off = align_up(off + p->stap_off.size() * sizeof(int));
  for (int s = 0; s < 2; ++s)
    for (int f = 0; f < 2; ++f) { p->o_state[s][f] = off; off = align_up(off + fb); }
  if (p->pml)
    for (int s = 0; s < 2; ++s)
      for (int f = 0; f < 2; ++f) { p->o_psi[s][f] = off; off = align_up(off + fb); }
  if (p->for_gradient) {
    for (int s = 0; s < 2; ++s)
      for (int f = 0; f < 2; ++f) { p->o_adj[s][f] = off; off = align_up(off + fb); }
    if (p->pml) {
      for (int s = 0; s < 2; ++s)
        for (int f = 0; f < 2; ++f) { p->o_apsi[s][f] = off; off = align_up(off + fb); }
      p->o_ckpsi = off;  // checkpoints 1..nseg-1, psi_x and psi_y each (float32)
      off = align_up(off + (size_t)(p->nseg - 1) * 2 * fb);
    }
    p->ckpt_elem_bytes = (t.ckpt_store == FDTD_STORE_F32) ? 4 : 2;
    const size_t nck = (size_t)(p->nseg - 1) * 2;  // checkpoints 1..nseg-1, two fields each
    p->o_ckpt = off; off = align_up(off + nck * p->field_elems * p->ckpt_elem_bytes);
    p->o_scales = off; off = align_up(off + nck * 2 * problem->n_shots * sizeof(float) + 16);
    // the recompute's segment buffer; with kept segments, one per kept segment (the
    // recompute reuses the first once the kept ones are imaged)
    p->o_seg = off; off = align_up(off + (size_t)std::max(1, p->kept) * p->ckpt_every * fb);
    // the adjoint's imaging sums sum w Q dt^2 / dy^2 (w = coef l), float64 (ny, pitch),
    // divided by coef once per pass into the caller's gradient
    p->o_graw = off; off = align_up(off + (size_t)g.ny * g.pitch * sizeof(double));
  }
  p->total = off;
  *out = p;
  return FDTD_OK;
}

int32_t fdtd_plan_destroy(fdtd_plan* plan) {
  delete plan;
  return FDTD_OK;
}

int32_t fdtd_plan_workspace_bytes(const fdtd_plan* plan, size_t* bytes) {
  if (!plan || !bytes) return fail(FDTD_ERR_INVALID, "null argument");
  *bytes = plan->total;
  return FDTD_OK;
}

int32_t fdtd_plan_tuning(const fdtd_plan* plan, fdtd_tuning* tuning) {
  if (!plan || !tuning) return fail(FDTD_ERR_INVALID, "null argument");
  *tuning = plan->tun;
  return FDTD_OK;
}

int32_t fdtd_plan_bind(fdtd_plan* p, void* workspace, size_t bytes, void* stream) {
  if (!p || !workspace) return fail(FDTD_ERR_WORKSPACE, "workspace missing");
  if (bytes < p->total) return fail(FDTD_ERR_WORKSPACE, "workspace too small: need " + std::to_string(p->total) + " bytes");
  if (reinterpret_cast<uintptr_t>(workspace) % ALIGN) return fail(FDTD_ERR_WORKSPACE, "workspace must be 256-byte aligned");
  cudaStream_t st = (cudaStream_t)stream;
  p->ws = reinterpret_cast<char*>(workspace);
  p->ws_bytes = bytes;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  e = cudaDeviceGetAttribute(&p->sm_count, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaDeviceGetAttribute");
  struct Up { size_t off; const void* src; size_t n; };
  const Up ups[] = {
      {p->o_tiles, p->tiles.data(), p->tiles.size() * sizeof(TbTile)},
      {p->o_taps, p->taps.data(), p->taps.size() * sizeof(TbTap)},
      {p->o_tmask, p->tmask.data(), p->tmask.size() * sizeof(TbMask)},
      {p->o_rxl, p->rxl.data(), p->rxl.size() * sizeof(int)},
      {p->o_recs, p->recs.data(), p->recs.size() * sizeof(TbRec)},
      {p->o_src, p->src.data(), p->src.size() * sizeof(SrcNode)},
      {p->o_stap, p->stap.data(), p->stap.size() * sizeof(SrcTap)},
      {p->o_stap_off, p->stap_off.data(), p->stap_off.size() * sizeof(int)},
  };
  for (const Up& u : ups) {
    if (!u.n) continue;
    e = cudaMemcpyAsync(p->ws + u.off, u.src, u.n, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return cuda_fail(e, "table upload");
  }
  if (p->pml) {
    // PML face fields start at zero and stay zero outside the PML tiles, which
    // never write there
    const size_t fb = p->field_elems * sizeof(float);
    std::vector<std::pair<size_t, size_t>> zero;
    for (int a = 0; a < 2; ++a)
      for (int f = 0; f < 2; ++f) {
        zero.push_back({p->o_psi[a][f], fb});
        if (p->for_gradient) zero.push_back({p->o_apsi[a][f], fb});
      }
    if (p->for_gradient) zero.push_back({p->o_ckpsi, (size_t)(p->nseg - 1) * 2 * fb});
    for (const auto& z : zero) {
      if (!z.second) continue;
      e = cudaMemsetAsync(p->ws + z.first, 0, z.second, st);
      if (e != cudaSuccess) return cuda_fail(e, "PML field clear");
    }
  }
  e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(e, "table upload sync");
  p->bound = true;
  p->have_ckpt = false;
  p->drop_graphs();
  return FDTD_OK;
}

int32_t fdtd_plan_set_medium(fdtd_plan* p, const float* coef, const float* mur,
                             const float* waveforms) {
  if (!p) return fail(FDTD_ERR_INVALID, "null plan");
  // The captured graphs read the medium through these pointers at run time: they
  // stay valid while the pointers do (an in-place update of the values), and are
  // captured again only when a pointer changes. Checkpoints of the old medium are
  // stale either way.
  const bool moved = (coef && coef != p->prob.grid.coef) || (mur && mur != p->prob.grid.mur) ||
                     (waveforms && waveforms != p->prob.src.waveforms);
  if (coef) p->prob.grid.coef = coef;
  if (mur) p->prob.grid.mur = mur;
  if (waveforms) p->prob.src.waveforms = waveforms;
  p->have_ckpt = false;
  if (moved) p->drop_graphs();
  return FDTD_OK;
}

}  // extern "C"

namespace {

// Runs `enqueue` on `st`, or replays it as a CUDA graph captured once per key.
template <typename F>
int32_t run_graphed(fdtd_plan* p, fdtd_plan::GraphSet& gs, const void* const (&key)[4], int flag,
                    cudaStream_t st, F enqueue) {
  if (p->tun.eager) return enqueue(st);
  fdtd_plan::Graph* found = nullptr;
  fdtd_plan::Graph* victim = &gs.slot[0];
  for (fdtd_plan::Graph& c : gs.slot) {
    bool hit = c.exec != nullptr && c.flag == flag;
    for (int i = 0; i < 4 && hit; ++i) hit = c.key[i] == key[i];
    if (hit) {
      found = &c;
      break;
    }
    if (!c.exec || (victim->exec && c.used < victim->used)) victim = &c;
  }
  const bool hit = found != nullptr;
  fdtd_plan::Graph& g = hit ? *found : *victim;
  g.used = ++p->graph_tick;
  if (!hit) {
    if (g.exec) cudaGraphExecDestroy(g.exec);
    g = fdtd_plan::Graph();
    g.used = p->graph_tick;
    cudaError_t e = cudaSuccess;
    if (!p->capture_stream) e = cudaStreamCreateWithFlags(&p->capture_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) return cuda_fail(e, "capture stream");
    // kernel attributes are set outside the capture
    for (int m = 0; m < 4; ++m) {
      if (m == MODE_FWDQ && p->kept == 0) continue;
      e = tb_configure(p->ky, m, p->nw, p->smem[m], p->pml != 0);
      if (e != cudaSuccess) return cuda_fail(e, "kernel attributes");
    }
    e = cudaStreamBeginCapture(p->capture_stream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return cuda_fail(e, "begin capture");
    const int32_t rc = enqueue(p->capture_stream);
    cudaGraph_t graph = nullptr;
    e = cudaStreamEndCapture(p->capture_stream, &graph);
    if (rc) {
      if (graph) cudaGraphDestroy(graph);
      return rc;
    }
    if (e != cudaSuccess) return cuda_fail(e, "end capture");
    e = cudaGraphInstantiate(&g.exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
      g.exec = nullptr;
      return cuda_fail(e, "graph instantiate");
    }
    for (int i = 0; i < 4; ++i) g.key[i] = key[i];
    g.flag = flag;
  }
  cudaError_t e = cudaGraphLaunch(g.exec, st);
  return e == cudaSuccess ? FDTD_OK : cuda_fail(e, "graph launch");
}

// One stream operation of a pass: a temporally blocked launch or a helper.
struct Op {
  enum Kind { LAUNCH, MEMSET, QUANT, DEQUANT, DIVIDE } kind = LAUNCH;
  int mode = 0;
  TbParams q;
  void* dst = nullptr;
  const void* src = nullptr;
  const float* aux = nullptr;  // QUANT: field subtracted from src; DEQUANT: base the value is subtracted from
  size_t bytes = 0;
  float* scales = nullptr;
  const float* cscales = nullptr;
  int n_shots = 0;
  long long per_shot = 0;
  int store = 0;
  double scale = 1.0;
};

int32_t exec_helper(const Op& op, cudaStream_t st) {
  cudaError_t e = cudaSuccess;
  if (op.kind == Op::MEMSET) e = cudaMemsetAsync(op.dst, 0, op.bytes, st);
  else if (op.kind == Op::QUANT)
    e = quantize_launch(static_cast<const float*>(op.src), op.aux, op.dst, op.scales, op.n_shots, op.per_shot,
                        op.store, st);
  else if (op.kind == Op::DEQUANT)
    e = dequantize_launch(op.src, op.cscales, op.aux, static_cast<float*>(op.dst), op.n_shots, op.per_shot,
                          op.store, st);
  else if (op.kind == Op::DIVIDE)
    e = grad_divide_launch(static_cast<const double*>(op.src), op.aux, op.scale, static_cast<double*>(op.dst),
                           op.per_shot, st);
  return e == cudaSuccess ? FDTD_OK : cuda_fail(e, "pass helper");
}

// Where a pass's operations go: straight onto a stream, or into a list (to be
// merged with other plans' passes into shared launches).
struct Sink {
  fdtd_plan* p;
  cudaStream_t st;
  std::vector<Op>* rec;
  int nsched = 0;  // item counters used so far in this pass
  int32_t emit(const Op& op) {
    if (rec) {
      rec->push_back(op);
      return FDTD_OK;
    }
    if (op.kind == Op::LAUNCH) {
      TbParams q = op.q;
      return launch(p, q, op.mode, st);
    }
    return exec_helper(op, st);
  }
  int32_t launch_tb(int mode, const TbParams& q) {
    Op op;
    op.kind = Op::LAUNCH;
    op.mode = mode;
    op.q = q;
    op.q.sched = nullptr;
    if (!rec) {  // a launch of its own (grouped launches deal items with a grid stride)
      if (nsched >= p->n_sched) return fail(FDTD_ERR_STATE, "item counters exhausted");
      op.q.sched = reinterpret_cast<int*>(p->ws + p->o_sched) + nsched++;
    }
    return emit(op);
  }
  // the pass's item counters start at zero
  int32_t reset_sched() { return memset(p->ws + p->o_sched, (size_t)p->n_sched * sizeof(int)); }
  int32_t memset(void* dst, size_t bytes) {
    Op op;
    op.kind = Op::MEMSET;
    op.dst = dst;
    op.bytes = bytes;
    return emit(op);
  }
  int32_t quant(const float* src, const float* minus, void* dst, float* scales, int n_shots, long long per_shot,
                int store) {
    Op op;
    op.kind = Op::QUANT;
    op.src = src;
    op.aux = minus;
    op.dst = dst;
    op.scales = scales;
    op.n_shots = n_shots;
    op.per_shot = per_shot;
    op.store = store;
    return emit(op);
  }
  // dst[i] += scale src[i] / coef[i] (nothing where coef is zero), float64, n elements
  int32_t divide(const double* src, const float* coef, double scale, double* dst, long long n) {
    Op op;
    op.kind = Op::DIVIDE;
    op.src = src;
    op.aux = coef;
    op.scale = scale;
    op.dst = dst;
    op.per_shot = n;
    return emit(op);
  }
  int32_t dequant(const void* src, const float* scales, const float* base, float* dst, int n_shots,
                  long long per_shot, int store) {
    Op op;
    op.kind = Op::DEQUANT;
    op.src = src;
    op.aux = base;
    op.cscales = scales;
    op.dst = dst;
    op.n_shots = n_shots;
    op.per_shot = per_shot;
    op.store = store;
    return emit(op);
  }
};

int32_t forward_enqueue(fdtd_plan* p, float* traces, float* u_prev_out, float* u_out,
                        int32_t save_checkpoints, Sink& k) {
  const size_t fb = p->field_elems * sizeof(float);
  int32_t rc0 = k.reset_sched();
  if (!rc0) rc0 = k.memset(p->ws + p->o_state[0][0], fb);
  if (!rc0) rc0 = k.memset(p->ws + p->o_state[0][1], fb);
  if (!rc0 && p->pml) rc0 = k.memset(p->ws + p->o_psi[0][0], fb);
  if (!rc0 && p->pml) rc0 = k.memset(p->ws + p->o_psi[0][1], fb);
  if (rc0) return rc0;
  TbParams q;
  fill_params(p, q);
  q.traces = traces;
  const int nt = p->prob.n_steps, T = p->tmax, C = p->ckpt_every;
  const float* in_prev = fptr(p, p->o_state[0][0]);
  const float* in_cur = fptr(p, p->o_state[0][1]);
  int in_set = 0;  // 0/1 = ping-pong set, -1 = elsewhere
  // PML face fields: their own ping-pong, written to the checkpoints at segment ends
  const float* in_px = p->pml ? fptr(p, p->o_psi[0][0]) : nullptr;
  const float* in_py = p->pml ? fptr(p, p->o_psi[0][1]) : nullptr;
  int psi_set = 0;
  // segments from kept0 on keep their stencil stream (no checkpoint at their starts)
  const int kept0 = save_checkpoints ? p->nseg - p->kept : p->nseg;
  for (int n0 = 0; n0 < nt; n0 += T) {
    const int ns = std::min(T, nt - n0), end = n0 + ns;
    const int out_set = (in_set == 0) ? 1 : 0;
    float* out_prev = fptr(p, p->o_state[out_set][0]);
    float* out_cur = fptr(p, p->o_state[out_set][1]);
    int next_set = out_set;
    const bool ckpt = save_checkpoints && end < nt && end % C == 0 && end / C < kept0;
    const int j = end / C;
    if (end == nt && u_out) {
      out_prev = u_prev_out;
      out_cur = u_out;
      next_set = -1;
    } else if (ckpt && p->tun.ckpt_store == FDTD_STORE_F32) {
      const size_t base = p->o_ckpt + (size_t)(j - 1) * 2 * fb;
      out_prev = fptr(p, base);
      out_cur = fptr(p, base + fb);
      next_set = -1;
    }
    q.in_prev = in_prev;
    q.in_cur = in_cur;
    q.out_prev = out_prev;
    q.out_cur = out_cur;
    q.n0 = n0;
    q.nsteps = ns;
    if (p->pml) {
      const int ps_out = (psi_set == 0) ? 1 : 0;
      q.in_psx = in_px;
      q.in_psy = in_py;
      if (ckpt) {
        q.out_psx = fptr(p, p->o_ckpsi + (size_t)(j - 1) * 2 * fb);
        q.out_psy = fptr(p, p->o_ckpsi + ((size_t)(j - 1) * 2 + 1) * fb);
        psi_set = -1;
      } else {
        q.out_psx = fptr(p, p->o_psi[ps_out][0]);
        q.out_psy = fptr(p, p->o_psi[ps_out][1]);
        psi_set = ps_out;
      }
      in_px = q.out_psx;
      in_py = q.out_psy;
    }
    int mode = MODE_FWD;
    if (n0 / C >= kept0) {  // a kept segment: its stream into its own buffer
      const int jq = n0 / C;
      mode = MODE_FWDQ;
      q.seg = fptr(p, p->o_seg + (size_t)(jq - kept0) * C * fb);
      q.seg_base = jq * C;
    }
    int32_t rc = k.launch_tb(mode, q);
    if (rc) return rc;
    if (ckpt && p->tun.ckpt_store != FDTD_STORE_F32) {
      const size_t eb = p->field_elems * p->ckpt_elem_bytes;
      const long long per_shot = (long long)p->prob.grid.ny * p->prob.grid.pitch;
      // slot 0: the step u - u_old, slot 1: u
      for (int f = 0; f < 2; ++f) {
        char* dst = p->ws + p->o_ckpt + ((size_t)(j - 1) * 2 + f) * eb;
        float* sc = fptr(p, p->o_scales) + ((size_t)(j - 1) * 2 + f) * 2 * p->prob.n_shots;
        rc = k.quant(out_cur, f == 0 ? out_prev : nullptr, dst, sc, p->prob.n_shots, per_shot, p->tun.ckpt_store);
        if (rc) return rc;
      }
    }
    in_prev = out_prev;
    in_cur = out_cur;
    in_set = next_set;
  }
  return FDTD_OK;
}

int32_t adjoint_enqueue(fdtd_plan* p, const float* residual, double* grad_c2, Sink& k) {
  const size_t fb = p->field_elems * sizeof(float);
  int32_t rc0 = k.reset_sched();
  if (!rc0) rc0 = k.memset(p->ws + p->o_adj[0][0], fb);
  if (!rc0) rc0 = k.memset(p->ws + p->o_adj[0][1], fb);
  if (!rc0 && p->pml) rc0 = k.memset(p->ws + p->o_apsi[0][0], fb);
  if (!rc0 && p->pml) rc0 = k.memset(p->ws + p->o_apsi[0][1], fb);
  if (rc0) return rc0;
  double* graw = reinterpret_cast<double*>(p->ws + p->o_graw);
  const long long cells = (long long)p->prob.grid.ny * p->prob.grid.pitch;
  rc0 = k.memset(graw, (size_t)cells * sizeof(double));
  if (rc0) return rc0;
  TbParams q;
  fill_params(p, q);
  q.residual = residual;
  q.grad = graw;
  // the segment buffer holds Q = dy^2 lap(u^{n-1}) (the recompute's stencil value):
  // dt^2 lap = dt^2 Q / dy^2
  q.scale = p->prob.grid.dt * p->prob.grid.dt / (p->prob.grid.dy * p->prob.grid.dy);
  q.seg = fptr(p, p->o_seg);
  const int nt = p->prob.n_steps, T = p->tmax, C = p->ckpt_every;
  const int kept0 = p->nseg - p->kept;  // segments from kept0 on were kept by the forward
  int adj_in = 0;
  const long long per_shot = (long long)p->prob.grid.ny * p->prob.grid.pitch;
  for (int j = p->nseg - 1; j >= 0; --j) {
    const int a = j * C, b = std::min(a + C, nt);
    if (j >= kept0) {  // a kept segment: the forward wrote its stream
      q.seg = fptr(p, p->o_seg + (size_t)(j - kept0) * C * fb);
      q.seg_base = a;
    } else {
      q.seg = fptr(p, p->o_seg);
      const float* in_prev;
      const float* in_cur;
      int in_set;
      // the forward's PML face fields at the segment start
      const float* in_px = nullptr;
      const float* in_py = nullptr;
      int psi_set = 0;
      if (p->pml) {
        if (j == 0) {
          int32_t rc = k.memset(p->ws + p->o_psi[0][0], fb);
          if (!rc) rc = k.memset(p->ws + p->o_psi[0][1], fb);
          if (rc) return rc;
          in_px = fptr(p, p->o_psi[0][0]);
          in_py = fptr(p, p->o_psi[0][1]);
        } else {
          in_px = fptr(p, p->o_ckpsi + (size_t)(j - 1) * 2 * fb);
          in_py = fptr(p, p->o_ckpsi + ((size_t)(j - 1) * 2 + 1) * fb);
          psi_set = -1;
        }
      }
      if (j == 0) {
        int32_t rc = k.memset(p->ws + p->o_state[0][0], fb);
        if (!rc) rc = k.memset(p->ws + p->o_state[0][1], fb);
        if (rc) return rc;
        in_prev = fptr(p, p->o_state[0][0]);
        in_cur = fptr(p, p->o_state[0][1]);
        in_set = 0;
      } else if (p->tun.ckpt_store == FDTD_STORE_F32) {
        const size_t base = p->o_ckpt + (size_t)(j - 1) * 2 * fb;
        in_prev = fptr(p, base);
        in_cur = fptr(p, base + fb);
        in_set = -1;
      } else {
        const size_t eb = p->field_elems * p->ckpt_elem_bytes;
        // u first (slot 1), then u_old = u - (u - u_old) (slot 0)
        for (int f = 1; f >= 0; --f) {
          const char* src = p->ws + p->o_ckpt + ((size_t)(j - 1) * 2 + f) * eb;
          const float* sc = fptr(p, p->o_scales) + ((size_t)(j - 1) * 2 + f) * 2 * p->prob.n_shots;
          const int32_t rc = k.dequant(src, sc, f == 0 ? fptr(p, p->o_state[0][1]) : nullptr,
                                       fptr(p, p->o_state[0][f]), p->prob.n_shots, per_shot, p->tun.ckpt_store);
          if (rc) return rc;
        }
        in_prev = fptr(p, p->o_state[0][0]);
        in_cur = fptr(p, p->o_state[0][1]);
        in_set = 0;
      }
      // recompute the segment, keeping lap(u^{n-1}) of every step n in [a, b)
      q.seg_base = a;
      for (int n0 = a; n0 < b; n0 += T) {
        const int ns = std::min(T, b - n0);
        const int out_set = (in_set == 0) ? 1 : 0;
        q.in_prev = in_prev;
        q.in_cur = in_cur;
        q.out_prev = fptr(p, p->o_state[out_set][0]);
        q.out_cur = fptr(p, p->o_state[out_set][1]);
        q.n0 = n0;
        q.nsteps = ns;
        if (p->pml) {
          const int ps_out = (psi_set == 0) ? 1 : 0;
          q.in_psx = in_px;
          q.in_psy = in_py;
          q.out_psx = fptr(p, p->o_psi[ps_out][0]);
          q.out_psy = fptr(p, p->o_psi[ps_out][1]);
          in_px = q.out_psx;
          in_py = q.out_psy;
          psi_set = ps_out;
        }
        int32_t rc = k.launch_tb(MODE_REC, q);
        if (rc) return rc;
        in_prev = q.out_prev;
        in_cur = q.out_cur;
        in_set = out_set;
      }
    }
    // reverse-time adjoint over the segment
    for (int ntop = b - 1; ntop >= a; ntop -= T) {
      const int ns = std::min(T, ntop - a + 1);
      const int out = adj_in ^ 1;
      q.in_prev = fptr(p, p->o_adj[adj_in][0]);
      q.in_cur = fptr(p, p->o_adj[adj_in][1]);
      q.out_prev = fptr(p, p->o_adj[out][0]);
      q.out_cur = fptr(p, p->o_adj[out][1]);
      q.n0 = ntop;
      q.nsteps = ns;
      if (p->pml) {  // the adjoint's own face fields (the same PML acts on w)
        q.in_psx = fptr(p, p->o_apsi[adj_in][0]);
        q.in_psy = fptr(p, p->o_apsi[adj_in][1]);
        q.out_psx = fptr(p, p->o_apsi[out][0]);
        q.out_psy = fptr(p, p->o_apsi[out][1]);
      }
      int32_t rc = k.launch_tb(MODE_ADJ, q);
      if (rc) return rc;
      adj_in = out;
    }
  }
  // grad_c2 += dt^2 lap-imaging = (dt^2 / dy^2) (sum w Q) / coef: the w = coef l form
  // divided out once
  return k.divide(graw, p->prob.grid.coef, q.scale, grad_c2, cells);
}

// ---- several plans in shared launches (uneven batches: grids of different
// sizes, steps and temporal-block depths, one launch shape)

struct GroupAction {
  int helper_plan = -1;      // >= 0: one helper op of that plan
  size_t helper_op = 0;
  int mode = 0;              // else: one shared launch of `members`
  std::vector<std::pair<int, size_t>> members;
};

size_t group_launch_bound(fdtd_plan* const* plans, int n) {
  size_t launches = 0;
  for (int i = 0; i < n; ++i) {
    const fdtd_plan* p = plans[i];
    const size_t per_pass = (size_t)(p->prob.n_steps + p->tmax - 1) / p->tmax;
    const size_t per_seg = (size_t)(p->ckpt_every + p->tmax - 1) / p->tmax;
    launches += std::max(per_pass, (size_t)p->nseg * 2 * per_seg);
  }
  return launches;
}

size_t group_bytes(fdtd_plan* const* plans, int n) {
  const size_t L = group_launch_bound(plans, n);
  return align_up(L * sizeof(TbParams)) + align_up(L * (size_t)(n + 1) * sizeof(int));
}

template <typename F>
int32_t group_run(fdtd_plan* const* plans, int n, void* workspace, size_t bytes, cudaStream_t st, F enqueue) {
  if (!plans || n < 1) return fail(FDTD_ERR_INVALID, "group: no plans");
  for (int i = 0; i < n; ++i) {
    if (!plans[i] || !plans[i]->bound) return fail(FDTD_ERR_STATE, "group: every plan must be bound");
    if (plans[i]->ky != plans[0]->ky || plans[i]->nw != plans[0]->nw)
      return fail(FDTD_ERR_UNSUPPORTED, "group: plans must share rows_per_lane and warps");
    if (plans[i]->pml) return fail(FDTD_ERR_UNSUPPORTED, "group: grids with a PML layer run as separate plans");
  }
  if (!workspace || bytes < group_bytes(plans, n)) return fail(FDTD_ERR_WORKSPACE, "group: workspace too small");
  // every plan's pass as a list of operations
  std::vector<std::vector<Op>> ops(n);
  for (int i = 0; i < n; ++i) {
    Sink k{plans[i], st, &ops[i]};
    const int32_t rc = enqueue(plans[i], k);
    if (rc) return rc;
  }
  // rounds: each plan runs its helpers up to its next launch; the next launches of
  // all plans form one shared launch per mode
  std::vector<size_t> idx(n, 0);
  std::vector<GroupAction> acts;
  for (;;) {
    bool left = false;
    for (int i = 0; i < n; ++i) {
      while (idx[i] < ops[i].size() && ops[i][idx[i]].kind != Op::LAUNCH) {
        GroupAction a;
        a.helper_plan = i;
        a.helper_op = idx[i]++;
        acts.push_back(a);
      }
      left = left || idx[i] < ops[i].size();
    }
    if (!left) break;
    for (int m = 0; m < 4; ++m) {
      GroupAction a;
      a.mode = m;
      for (int i = 0; i < n; ++i)
        if (idx[i] < ops[i].size() && ops[i][idx[i]].mode == m) a.members.push_back({i, idx[i]});
      if (a.members.empty()) continue;
      for (auto& mb : a.members) ++idx[mb.first];
      acts.push_back(a);
    }
  }
  // parameters and item offsets of the shared launches, uploaded at once
  std::vector<TbParams> hp;
  std::vector<int> hoff;
  for (const GroupAction& a : acts) {
    if (a.helper_plan >= 0 || a.members.size() < 2) continue;
    int items = 0;
    for (auto& mb : a.members) {
      hp.push_back(ops[mb.first][mb.second].q);
      hoff.push_back(items);
      items += plans[mb.first]->prob.n_shots * (int)plans[mb.first]->tiles.size();
    }
    hoff.push_back(items);
  }
  const size_t L = group_launch_bound(plans, n);
  if (hp.size() > L || hoff.size() > L * (size_t)(n + 1)) return fail(FDTD_ERR_UNSUPPORTED, "group: launch bound exceeded");
  char* dws = static_cast<char*>(workspace);
  TbParams* dparams = reinterpret_cast<TbParams*>(dws);
  int* doff = reinterpret_cast<int*>(dws + align_up(L * sizeof(TbParams)));
  cudaError_t e = cudaSuccess;
  if (!hp.empty()) e = cudaMemcpyAsync(dparams, hp.data(), hp.size() * sizeof(TbParams), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess && !hoff.empty())
    e = cudaMemcpyAsync(doff, hoff.data(), hoff.size() * sizeof(int), cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return cuda_fail(e, "group parameter upload");
  size_t pk = 0, ok = 0;
  for (const GroupAction& a : acts) {
    if (a.helper_plan >= 0) {
      const int32_t rc = exec_helper(ops[a.helper_plan][a.helper_op], st);
      if (rc) return rc;
      continue;
    }
    if (a.members.size() == 1) {
      fdtd_plan* p = plans[a.members[0].first];
      TbParams q = ops[a.members[0].first][a.members[0].second].q;
      const int32_t rc = launch(p, q, a.mode, st);
      if (rc) return rc;
      continue;
    }
    size_t smem = 0;
    int items = 0;
    bool adj_coef = true;  // every member keeps its adjoint coefficient tile in shared memory
    for (auto& mb : a.members) {
      smem = std::max(smem, plans[mb.first]->smem[a.mode]);
      items += plans[mb.first]->prob.n_shots * (int)plans[mb.first]->tiles.size();
      adj_coef = adj_coef && plans[mb.first]->adj_coef;
    }
    if (smem + tb_group_static_smem() > 232448) return fail(FDTD_ERR_UNSUPPORTED, "group: shared memory need exceeds 227 KB");
    TbGroup g;
    g.params = dparams + pk;
    g.item_off = doff + ok;
    g.nplans = (int)a.members.size();
    g.nitems = items;
    const int grid = std::max(1, std::min(items, plans[0]->sm_count * std::max(1, plans[0]->tun.ctas_per_sm)));
    e = tb_group_launch(g, plans[0]->ky, plans[0]->nw, a.mode, adj_coef, grid, smem, st);
    if (e != cudaSuccess) return cuda_fail(e, "grouped kernel launch");
    pk += a.members.size();
    ok += a.members.size() + 1;
  }
  return FDTD_OK;
}

}  // namespace

extern "C" {

size_t fdtd_group_workspace_bytes(fdtd_plan* const* plans, int32_t n) {
  if (!plans || n < 1) return 0;
  for (int i = 0; i < n; ++i)
    if (!plans[i]) return 0;
  return group_bytes(plans, n);
}

int32_t fdtd_group_forward(fdtd_plan* const* plans, int32_t n, float* const* traces, int32_t save_checkpoints,
                           void* workspace, size_t bytes, void* stream) {
  if (!traces) return fail(FDTD_ERR_INVALID, "group: traces must be set");
  for (int i = 0; i < n; ++i) {
    if (!traces[i]) return fail(FDTD_ERR_INVALID, "group: traces must be set");
    if (plans && plans[i] && save_checkpoints && !plans[i]->for_gradient)
      return fail(FDTD_ERR_STATE, "group: a plan was created without gradient storage");
  }
  int k = 0;
  const int32_t rc = group_run(plans, n, workspace, bytes, (cudaStream_t)stream, [&](fdtd_plan* p, Sink& s) {
    return forward_enqueue(p, traces[k++], nullptr, nullptr, save_checkpoints, s);
  });
  if (rc) return rc;
  for (int i = 0; i < n; ++i) plans[i]->have_ckpt = save_checkpoints != 0;
  return FDTD_OK;
}

int32_t fdtd_group_adjoint(fdtd_plan* const* plans, int32_t n, const float* const* residuals, double* const* grads,
                           void* workspace, size_t bytes, void* stream) {
  if (!residuals || !grads) return fail(FDTD_ERR_INVALID, "group: residuals and gradients must be set");
  for (int i = 0; i < n; ++i) {
    if (!residuals[i] || !grads[i]) return fail(FDTD_ERR_INVALID, "group: residuals and gradients must be set");
    if (plans && plans[i] && !plans[i]->have_ckpt) return fail(FDTD_ERR_STATE, "group: run the forward with checkpoints first");
  }
  int k = 0;
  return group_run(plans, n, workspace, bytes, (cudaStream_t)stream, [&](fdtd_plan* p, Sink& s) {
    const int j = k++;
    return adjoint_enqueue(p, residuals[j], grads[j], s);
  });
}

int32_t fdtd_forward(fdtd_plan* p, float* traces, float* u_prev_out, float* u_out,
                     int32_t save_checkpoints, void* stream) {
  if (!p || !p->bound) return fail(FDTD_ERR_STATE, "plan is not bound to a workspace");
  if (!traces) return fail(FDTD_ERR_INVALID, "traces must be set");
  if ((u_prev_out == nullptr) != (u_out == nullptr)) return fail(FDTD_ERR_INVALID, "give both final-state outputs or neither");
  if (save_checkpoints && !p->for_gradient) return fail(FDTD_ERR_STATE, "plan was created without gradient storage");
  const void* const key[4] = {traces, u_prev_out, u_out, nullptr};
  const int32_t rc = run_graphed(p, p->g_fwd, key, save_checkpoints != 0, (cudaStream_t)stream,
                                 [&](cudaStream_t st) {
                                   Sink k{p, st, nullptr};
                                   return forward_enqueue(p, traces, u_prev_out, u_out, save_checkpoints, k);
                                 });
  if (rc) return rc;
  p->have_ckpt = save_checkpoints != 0;
  return FDTD_OK;
}

int32_t fdtd_adjoint(fdtd_plan* p, const float* residual, double* grad_c2, void* stream) {
  if (!p || !p->bound) return fail(FDTD_ERR_STATE, "plan is not bound to a workspace");
  if (!p->have_ckpt) return fail(FDTD_ERR_STATE, "run fdtd_forward with save_checkpoints first");
  if (!residual || !grad_c2) return fail(FDTD_ERR_INVALID, "null pointer");
  const void* const key[4] = {residual, grad_c2, nullptr, nullptr};
  return run_graphed(p, p->g_adj, key, 0, (cudaStream_t)stream,
                     [&](cudaStream_t st) {
                       Sink k{p, st, nullptr};
                       return adjoint_enqueue(p, residual, grad_c2, k);
                     });
}

// ----------------------------------------------------------- plain engine

size_t fdtd_forward_plain_workspace(const fdtd_problem* prob) {
  if (!prob) return 0;
  const size_t plane = (size_t)prob->grid.ny * prob->grid.pitch * sizeof(float);
  const size_t R = prob->rx.n;
  const size_t K = prob->src.per_shot > 0 ? prob->src.per_shot : 0;
  return align_up(3 * plane) + align_up(R * 2 * sizeof(int32_t)) + align_up(R * 4 * sizeof(float)) +
         align_up((size_t)prob->n_shots * K * (3 * sizeof(int32_t) + sizeof(float)) + 16);
}

}  // extern "C"

namespace {

int32_t forward_plain_impl(const fdtd_problem* prob, const fdtd_density* density, float* traces, void* workspace,
                           size_t bytes, void* stream) {
  if (!prob || !traces) return fail(FDTD_ERR_INVALID, "null argument");
  int32_t rc = validate_plain_problem(*prob);
  if (rc) return rc;
  if (!workspace || bytes < fdtd_forward_plain_workspace(prob)) return fail(FDTD_ERR_WORKSPACE, "workspace too small");
  cudaStream_t st = (cudaStream_t)stream;
  const fdtd_grid& g = prob->grid;
  const size_t plane = (size_t)g.ny * g.pitch;
  const int R = prob->rx.n, S = prob->n_shots, nt = prob->n_steps;
  const int K = prob->src.per_shot > 0 ? prob->src.per_shot : 0;
  char* w = reinterpret_cast<char*>(workspace);
  float* f[3] = {reinterpret_cast<float*>(w), reinterpret_cast<float*>(w) + plane,
                 reinterpret_cast<float*>(w) + 2 * plane};
  size_t off = align_up(3 * plane * sizeof(float));
  int32_t* rx_rc = reinterpret_cast<int32_t*>(w + off);
  off += align_up((size_t)R * 2 * sizeof(int32_t));
  float* rx_w = reinterpret_cast<float*>(w + off);
  off += align_up((size_t)R * 4 * sizeof(float));
  int32_t* s_row = reinterpret_cast<int32_t*>(w + off);
  int32_t* s_col = s_row + (size_t)S * K;
  int32_t* s_wave = s_col + (size_t)S * K;
  float* s_w = reinterpret_cast<float*>(s_wave + (size_t)S * K);
  std::vector<int32_t> rc_h(2 * (size_t)R);
  for (int r = 0; r < R; ++r) { rc_h[2 * r] = prob->rx.row0[r]; rc_h[2 * r + 1] = prob->rx.col0[r]; }
  cudaError_t e = cudaMemcpyAsync(rx_rc, rc_h.data(), rc_h.size() * sizeof(int32_t), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(rx_w, prob->rx.w, (size_t)R * 4 * sizeof(float), cudaMemcpyHostToDevice, st);
  if (K > 0) {
    if (e == cudaSuccess) e = cudaMemcpyAsync(s_row, prob->src.row, (size_t)S * K * 4, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(s_col, prob->src.col, (size_t)S * K * 4, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(s_wave, prob->src.wave, (size_t)S * K * 4, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(s_w, prob->src.w, (size_t)S * K * 4, cudaMemcpyHostToDevice, st);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(e, "plain forward upload");
  for (int s = 0; s < S; ++s) {
    e = cudaMemsetAsync(w, 0, 3 * plane * sizeof(float), st);
    if (e != cudaSuccess) return cuda_fail(e, "plain forward reset");
    int io = 0, ic = 1, in = 2;
    for (int n = 0; n < nt; ++n) {
      rc = step_impl(&g, density, 1, f[io], f[ic], f[in], K, s_row + (size_t)s * K, s_col + (size_t)s * K,
                     s_w + (size_t)s * K, s_wave + (size_t)s * K, prob->src.waveforms,
                     prob->src.waveform_len, n, nullptr, 0, stream);
      if (rc) return rc;
      e = gather_launch(g.ny, g.pitch, 1, f[in], R, rx_rc, rx_w, traces + (size_t)s * R * nt + n, 0, nt, st);
      if (e != cudaSuccess) return cuda_fail(e, "plain gather");
      const int t = io; io = ic; ic = in; in = t;
    }
  }
  return FDTD_OK;
}

}  // namespace

extern "C" {

int32_t fdtd_forward_plain(const fdtd_problem* prob, float* traces, void* workspace, size_t bytes,
                           void* stream) {
  return forward_plain_impl(prob, nullptr, traces, workspace, bytes, stream);
}

int32_t fdtd_forward_plain_density(const fdtd_problem* prob, const fdtd_density* density, float* traces,
                                   void* workspace, size_t bytes, void* stream) {
  if (!density) return fail(FDTD_ERR_INVALID, "null density");
  return forward_plain_impl(prob, density, traces, workspace, bytes, stream);
}

size_t fdtd_gradient_plain_workspace(const fdtd_problem* prob) {
  if (!prob) return 0;
  const size_t plane = (size_t)prob->grid.ny * prob->grid.pitch * sizeof(float);
  const size_t R = prob->rx.n, nt = prob->n_steps;
  return fdtd_forward_plain_workspace(prob) + align_up((nt + 2) * plane) + align_up(4 * plane) +
         align_up(2 * R * nt * sizeof(float)) + align_up(4 * R * (10 + 8) * sizeof(int32_t));
}

}  // extern "C"

namespace {

// The plain per-shot gradient; with `density` the variable-density operator, the
// adjoint in the reference's l form and the imaging into g_kappa (grad_c2) and the
// face gradients g_bx (ny, pitch + 4), g_by (ny + 1, pitch).
int32_t gradient_plain_impl(const fdtd_problem* prob, const fdtd_density* density, const float* observed,
                            const int32_t* mute, double* misfit, double* grad_c2, double* g_bx, double* g_by,
                            void* workspace, size_t bytes, void* stream) {
  if (!prob || !observed || !misfit || !grad_c2) return fail(FDTD_ERR_INVALID, "null argument");
  if (density && (!g_bx || !g_by)) return fail(FDTD_ERR_INVALID, "face gradients missing");
  int32_t rc = validate_plain_problem(*prob);
  if (rc) return rc;
  if (!workspace || bytes < fdtd_gradient_plain_workspace(prob)) return fail(FDTD_ERR_WORKSPACE, "workspace too small");
  cudaStream_t st = (cudaStream_t)stream;
  const fdtd_grid& g = prob->grid;
  const size_t plane = (size_t)g.ny * g.pitch;
  const int R = prob->rx.n, S = prob->n_shots, nt = prob->n_steps;
  const int K = prob->src.per_shot > 0 ? prob->src.per_shot : 0;
  char* w = reinterpret_cast<char*>(workspace);
  // shared pieces: receivers and sources (same layout as the plain forward)
  size_t off = align_up(3 * plane * sizeof(float));
  int32_t* rx_rc = reinterpret_cast<int32_t*>(w + off);
  off += align_up((size_t)R * 2 * sizeof(int32_t));
  float* rx_w = reinterpret_cast<float*>(w + off);
  off += align_up((size_t)R * 4 * sizeof(float));
  int32_t* s_row = reinterpret_cast<int32_t*>(w + off);
  int32_t* s_col = s_row + (size_t)S * K;
  int32_t* s_wave = s_col + (size_t)S * K;
  float* s_w = reinterpret_cast<float*>(s_wave + (size_t)S * K);
  off = fdtd_forward_plain_workspace(prob);
  float* hist = reinterpret_cast<float*>(w + off);  // two zero planes, then u after every step
  off += align_up((size_t)(nt + 2) * plane * sizeof(float));
  float* lam = reinterpret_cast<float*>(w + off);   // three adjoint planes + the dense scatter plane
  off += align_up(4 * plane * sizeof(float));
  float* trace = reinterpret_cast<float*>(w + off);
  float* resid = trace + (size_t)R * nt;
  off += align_up(2 * (size_t)R * nt * sizeof(float));
  int32_t* tap_nodes = reinterpret_cast<int32_t*>(w + off);
  float* tap_w = reinterpret_cast<float*>(tap_nodes + (size_t)4 * R * 10);
  std::vector<int32_t> nodes_h((size_t)4 * R * 10);
  std::vector<float> tw_h((size_t)4 * R * 8);
  int32_t n_nodes = 4 * R;
  rc = fdtd_tap_table(g.ny, g.nx, &prob->rx, nodes_h.data(), tw_h.data(), &n_nodes);
  if (rc) return rc;
  std::vector<int32_t> rc_h(2 * (size_t)R);
  for (int r = 0; r < R; ++r) { rc_h[2 * r] = prob->rx.row0[r]; rc_h[2 * r + 1] = prob->rx.col0[r]; }
  cudaError_t e = cudaMemcpyAsync(rx_rc, rc_h.data(), rc_h.size() * 4, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(rx_w, prob->rx.w, (size_t)R * 16, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(tap_nodes, nodes_h.data(), (size_t)n_nodes * 40, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(tap_w, tw_h.data(), (size_t)n_nodes * 32, cudaMemcpyHostToDevice, st);
  if (K > 0) {
    if (e == cudaSuccess) e = cudaMemcpyAsync(s_row, prob->src.row, (size_t)S * K * 4, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(s_col, prob->src.col, (size_t)S * K * 4, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(s_wave, prob->src.wave, (size_t)S * K * 4, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(s_w, prob->src.w, (size_t)S * K * 4, cudaMemcpyHostToDevice, st);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(e, "plain gradient upload");
  const double idx2 = 1.0 / (g.dx * g.dx), idy2 = 1.0 / (g.dy * g.dy);
  float* dense = lam + 3 * plane;
  for (int s = 0; s < S; ++s) {
    // forward with the whole history: hist[k + 2] holds u after step k
    e = cudaMemsetAsync(hist, 0, 2 * plane * sizeof(float), st);
    if (e != cudaSuccess) return cuda_fail(e, "plain gradient reset");
    for (int n = 0; n < nt; ++n) {
      float* un = hist + (size_t)(n + 2) * plane;
      rc = step_impl(&g, density, 1, hist + (size_t)n * plane, hist + (size_t)(n + 1) * plane, un, K,
                     s_row + (size_t)s * K, s_col + (size_t)s * K, s_w + (size_t)s * K,
                     s_wave + (size_t)s * K, prob->src.waveforms, prob->src.waveform_len, n,
                     nullptr, 0, stream);
      if (rc) return rc;
      e = gather_launch(g.ny, g.pitch, 1, un, R, rx_rc, rx_w, trace + n, 0, nt, st);
      if (e != cudaSuccess) return cuda_fail(e, "plain gather");
    }
    e = residual_launch(1, R, nt, trace, observed + (size_t)s * R * nt, 0, mute ? mute + s : nullptr,
                        resid, misfit, st);
    if (e != cudaSuccess) return cuda_fail(e, "plain residual");
    // reverse-time adjoint, one scatter + step + image launch per step
    e = cudaMemsetAsync(lam, 0, 4 * plane * sizeof(float), st);
    if (e != cudaSuccess) return cuda_fail(e, "plain adjoint reset");
    int io = 0, ic = 1, in = 2;
    for (int n = nt - 1; n >= 0; --n) {
      e = scatter_launch(g.ny, g.pitch, 1, n_nodes, tap_nodes, tap_w, resid + n, 0, nt, dense, st);
      if (e != cudaSuccess) return cuda_fail(e, "plain scatter");
      // the adjoint in w = coef * l form, as the fused engine carries it; with
      // variable density in the reference's l form
      rc = step_impl(&g, density, 1, lam + (size_t)io * plane, lam + (size_t)ic * plane, lam + (size_t)in * plane,
                     0, nullptr, nullptr, nullptr, nullptr, nullptr, 0, 0, dense, density ? 1 : 2, stream);
      if (rc) return rc;
      if (n >= 1 && density) {
        e = image_density_launch(g.ny, g.nx, g.pitch, (float)idx2, (float)idy2, 1, lam + (size_t)in * plane,
                                 hist + (size_t)(n + 1) * plane, density->kappa, density->bx, density->by,
                                 g.dt * g.dt, g.dt * g.dt, grad_c2, g_bx, g_by, st);
        if (e != cudaSuccess) return cuda_fail(e, "plain density image");
      } else if (n >= 1) {
        e = image_launch(g.ny, g.nx, g.pitch, (float)idx2, (float)idy2, (float)(-2.0 * (idx2 + idy2)), 1,
                         lam + (size_t)in * plane, hist + (size_t)(n + 1) * plane, g.dt * g.dt, g.coef,
                         grad_c2, st);
        if (e != cudaSuccess) return cuda_fail(e, "plain image");
      }
      const int t = io; io = ic; ic = in; in = t;
    }
  }
  return FDTD_OK;
}

}  // namespace

extern "C" {

int32_t fdtd_gradient_plain(const fdtd_problem* prob, const float* observed, const int32_t* mute,
                            double* misfit, double* grad_c2, void* workspace, size_t bytes,
                            void* stream) {
  return gradient_plain_impl(prob, nullptr, observed, mute, misfit, grad_c2, nullptr, nullptr, workspace, bytes,
                             stream);
}

int32_t fdtd_gradient_plain_density(const fdtd_problem* prob, const fdtd_density* density, const float* observed,
                                    const int32_t* mute, double* misfit, double* g_kappa, double* g_bx,
                                    double* g_by, void* workspace, size_t bytes, void* stream) {
  if (!density) return fail(FDTD_ERR_INVALID, "null density");
  return gradient_plain_impl(prob, density, observed, mute, misfit, g_kappa, g_bx, g_by, workspace, bytes, stream);
}

}  // extern "C"
