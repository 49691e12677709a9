/*
 * fdtd_oracle.c -- float64 C restatement of the reference's fdtd2d forward and
 * adjoint-state gradient: TEST INFRASTRUCTURE ONLY.
 *
 * The same algorithm as oracle/fdtd_oracle.py (which is pinned to outputs of the
 * reference itself), written as plain loops so that the tests can run it at the
 * benchmark configurations' full sizes (512^2 x 4000 steps, 1024^2 x 6000 steps)
 * on the host cores in seconds per shot. Only tests/, __graft_entry__.smoke() and
 * bench.py's CPU legs load it, as the checker; the product never does.
 *
 * One call runs one shot; callers run shots in parallel threads (ctypes releases
 * the GIL during the call). Arrays are row-major (ny, nx), row = y, column = x.
 * Forward step, following fdtd2d/torch_backend.py:493-522 and 477-490:
 *   u+ = 2 u - u- + dt^2 c^2 lap(u)            (zero-padded 5-point Laplacian,
 *                                              torch_backend.py:122-132)
 *   u+[row_k, col_k] += w_k * wave[step]        (soft sources, torch_backend.py:517;
 *                                              desmond/src/phase2_numerics.py:107-118)
 *   Mur: left / right columns on rows 1..ny-2, bottom / top rows on columns
 *   1..nx-2 from the same u+, then the four corners as the mean of the x- and
 *   y-direction updates (fdtd2d/solver.py:90-124)
 *   traces[r, step] = bilinear sample of u+ (torch_backend.py:540-548)
 * Adjoint step (torch_backend.py:525-537, 563-598; invert_ring.py:683-701):
 *   l+ = 2 l - l- + dt^2 lap(c^2 l) + scatter(residual[:, n]), the forward's Mur,
 *   and for n >= 1  g += dt^2 l+ lap(u after step n-1).
 * With pml > 0 (no reference counterpart) the grid is padded by a PML layer of
 * that many cells (oracle/fdtd_oracle.py pml_step) instead of Mur edges; the
 * adjoint then runs as w = (c dt)^2 l with the same PML step.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
  int ny, nx;
  size_t W, n;               /* padded row length and field size: one zero cell all round */
  double idx2, idy2, diag, dt2;
  double* k2;                /* dt^2 c^2 (padded) */
  double* c2;                /* c^2 (padded) */
  double* kl; double* kr;    /* Mur k of the left / right column, per row */
  double* kb; double* kt;    /* Mur k of the bottom / top row, per column */
  double kcx[4], kcy[4];
  int cy[4], cx[4], iy[4], ix[4];
  /* PML (pml > 0 cells on every side of the grid; then no Mur edges, a rigid
     outer wall): 1-D damping tables and the per-cell update factors */
  int pml;
  double *sxc, *sxf, *axf, *bxf;  /* per column: sigma_x at the centre / left face, psi_x decay, forcing scale */
  double *syc, *syf, *ayf, *byf;  /* per row, the same for y */
  double *K, *A, *M;              /* padded: q (c dt)^2, q (2 - dt^2 sx sy), (1 - a) q */
} Medium;

#define AT(m, f, y, x) ((f)[((size_t)(y) + 1) * (m)->W + (size_t)(x) + 1])

static double mur1(double k, double u_in, double un_in, double u_edge) {
  return u_in + k * (un_in - u_edge);
}

static void medium_free(Medium* m) {
  free(m->k2);
  free(m->kl);
  free(m->sxc);
  free(m->K);
}

static int medium_init(Medium* m, int ny, int nx, double dx, double dy, double dt, const double* c) {
  memset(m, 0, sizeof(*m));
  m->ny = ny;
  m->nx = nx;
  m->W = (size_t)nx + 2;
  m->n = ((size_t)ny + 2) * m->W;
  m->idx2 = 1.0 / (dx * dx);
  m->idy2 = 1.0 / (dy * dy);
  m->diag = -2.0 * (m->idx2 + m->idy2);
  m->dt2 = dt * dt;
  m->k2 = (double*)calloc(2 * m->n, sizeof(double));
  m->kl = (double*)malloc(sizeof(double) * (2 * (size_t)ny + 2 * (size_t)nx));
  if (!m->k2 || !m->kl) { medium_free(m); return 2; }
  m->c2 = m->k2 + m->n;
  m->kr = m->kl + ny;
  m->kb = m->kr + ny;
  m->kt = m->kb + nx;
  for (int y = 0; y < ny; ++y)
    for (int x = 0; x < nx; ++x) {
      const double cc = c[(size_t)y * nx + x];
      AT(m, m->c2, y, x) = cc * cc;
      AT(m, m->k2, y, x) = m->dt2 * (cc * cc);
    }
  /* Mur coefficients (c dt - h) / (c dt + h) of the edge cells (torch_backend.py:264-275) */
#define MURK(cc, h) (((cc) * dt - (h)) / ((cc) * dt + (h)))
  for (int y = 0; y < ny; ++y) {
    m->kl[y] = MURK(c[(size_t)y * nx], dx);
    m->kr[y] = MURK(c[(size_t)y * nx + nx - 1], dx);
  }
  for (int x = 0; x < nx; ++x) {
    m->kb[x] = MURK(c[x], dy);
    m->kt[x] = MURK(c[(size_t)(ny - 1) * nx + x], dy);
  }
  const int cy[4] = {0, 0, ny - 1, ny - 1}, cx[4] = {0, nx - 1, 0, nx - 1};
  const int iy[4] = {1, 1, ny - 2, ny - 2}, ix[4] = {1, nx - 2, 1, nx - 2};
  for (int q = 0; q < 4; ++q) {
    const double cc = c[(size_t)cy[q] * nx + cx[q]];
    m->kcx[q] = MURK(cc, dx);
    m->kcy[q] = MURK(cc, dy);
    m->cy[q] = cy[q]; m->cx[q] = cx[q]; m->iy[q] = iy[q]; m->ix[q] = ix[q];
  }
#undef MURK
  return 0;
}

/* 5-point Laplacian of the padded field f at interior cell (row pointer, x) */
static inline double lap_at(const Medium* m, const double* row, int x) {
  const long W = (long)m->W;
  return (row[x - 1] + row[x + 1]) * m->idx2 + (row[x - W] + row[x + W]) * m->idy2 + m->diag * row[x];
}

/* PML tables (oracle/fdtd_oracle.py pml_coefficients): sigma = smax (depth / P)^2
   with smax = 3 c_max ln(1 / R) / (2 P h); depth measured from the layer's inner
   face, at cell centres and at left / bottom faces. */
static double pml_sigma(double x, int n, int P, double smax) {
  double lo = (P - 0.5) - x, hi = x - (n - P - 0.5), d = lo > hi ? lo : hi;
  if (d < 0.0) d = 0.0;
  return smax * (d / P) * (d / P);
}

static int medium_pml(Medium* m, const double* c, double dx, double dy, double dt, int P, double R) {
  const int ny = m->ny, nx = m->nx;
  double cmax = 0.0;
  for (size_t i = 0; i < (size_t)ny * nx; ++i) cmax = c[i] > cmax ? c[i] : cmax;
  const double smx = 3.0 * cmax * log(1.0 / R) / (2.0 * P * dx);
  const double smy = 3.0 * cmax * log(1.0 / R) / (2.0 * P * dy);
  m->pml = P;
  m->sxc = (double*)calloc(4 * (size_t)nx + 4 * (size_t)ny, sizeof(double));
  m->K = (double*)calloc(3 * m->n, sizeof(double));
  if (!m->sxc || !m->K) return 2;
  m->sxf = m->sxc + nx; m->axf = m->sxf + nx; m->bxf = m->axf + nx;
  m->syc = m->bxf + nx; m->syf = m->syc + ny; m->ayf = m->syf + ny; m->byf = m->ayf + ny;
  m->A = m->K + m->n; m->M = m->A + m->n;
  for (int i = 0; i < nx; ++i) {
    m->sxc[i] = pml_sigma(i, nx, P, smx);
    m->sxf[i] = pml_sigma(i - 0.5, nx, P, smx);
    m->axf[i] = (1.0 - 0.5 * dt * m->sxf[i]) / (1.0 + 0.5 * dt * m->sxf[i]);
    m->bxf[i] = dt / (dx * dx * (1.0 + 0.5 * dt * m->sxf[i]));
  }
  for (int j = 0; j < ny; ++j) {
    m->syc[j] = pml_sigma(j, ny, P, smy);
    m->syf[j] = pml_sigma(j - 0.5, ny, P, smy);
    m->ayf[j] = (1.0 - 0.5 * dt * m->syf[j]) / (1.0 + 0.5 * dt * m->syf[j]);
    m->byf[j] = dt / (dy * dy * (1.0 + 0.5 * dt * m->syf[j]));
  }
  for (int j = 0; j < ny; ++j)
    for (int i = 0; i < nx; ++i) {
      const double a = 0.5 * dt * (m->sxc[i] + m->syc[j]);
      const double q = 1.0 / (1.0 + a);
      AT(m, m->K, j, i) = q * AT(m, m->k2, j, i);
      AT(m, m->A, j, i) = q * (2.0 - dt * dt * m->sxc[i] * m->syc[j]);
      AT(m, m->M, j, i) = (1.0 - a) * q;
    }
  return 0;
}

/* One PML step of field f (forward: f = u; adjoint in w-form: f = (c dt)^2 l):
   face fields first (trapezoidal decay, forced by the differences of f across each
   face), then fn = K (lap f + div psi) + A f - M fo. psi beyond the grid is zero. */
static void step_pml(const Medium* m, const double* fo, const double* f, double* fn, const double* psx,
                     const double* psy, double* psxn, double* psyn) {
  const int ny = m->ny, nx = m->nx;
  const long W = (long)m->W;
  for (int y = 0; y < ny; ++y) {
    const double* fr = &AT(m, f, y, 0);
    for (int x = 0; x < nx; ++x) {
      AT(m, psxn, y, x) = m->axf[x] * AT(m, psx, y, x) + (m->syc[y] - m->sxf[x]) * m->bxf[x] * (fr[x] - fr[x - 1]);
      AT(m, psyn, y, x) = m->ayf[y] * AT(m, psy, y, x) + (m->sxc[x] - m->syf[y]) * m->byf[y] * (fr[x] - fr[x - W]);
    }
  }
  for (int y = 0; y < ny; ++y) {
    const double* fr = &AT(m, f, y, 0);
    const double* fo_r = &AT(m, fo, y, 0);
    double* out = &AT(m, fn, y, 0);
    for (int x = 0; x < nx; ++x) {
      const double px_r = (x + 1 < nx) ? AT(m, psxn, y, x + 1) : 0.0;
      const double py_t = (y + 1 < ny) ? AT(m, psyn, y + 1, x) : 0.0;
      const double div = (px_r - AT(m, psxn, y, x)) + (py_t - AT(m, psyn, y, x));
      out[x] = AT(m, m->K, y, x) * (lap_at(m, fr, x) + div) + (AT(m, m->A, y, x) * fr[x] - AT(m, m->M, y, x) * fo_r[x]);
    }
  }
}

/* un = 2 u - uo + dt^2 c^2 lap(u) */
static void step_forward(const Medium* m, const double* uo, const double* u, double* un) {
  for (int y = 0; y < m->ny; ++y) {
    const double* ur = &AT(m, u, y, 0);
    const double* po = &AT(m, uo, y, 0);
    const double* kk = &AT(m, m->k2, y, 0);
    double* out = &AT(m, un, y, 0);
    for (int x = 0; x < m->nx; ++x) out[x] = 2.0 * ur[x] - po[x] + kk[x] * lap_at(m, ur, x);
  }
}

/* ln = 2 l - lo + dt^2 lap(c^2 l); tmp is a padded scratch field (zero border) */
static void step_adjoint(const Medium* m, const double* lo, const double* l, double* ln, double* tmp) {
  for (int y = 0; y < m->ny; ++y) {
    const double* lr = &AT(m, l, y, 0);
    const double* cc = &AT(m, m->c2, y, 0);
    double* t = &AT(m, tmp, y, 0);
    for (int x = 0; x < m->nx; ++x) t[x] = cc[x] * lr[x];
  }
  for (int y = 0; y < m->ny; ++y) {
    const double* lr = &AT(m, l, y, 0);
    const double* po = &AT(m, lo, y, 0);
    const double* t = &AT(m, tmp, y, 0);
    double* out = &AT(m, ln, y, 0);
    for (int x = 0; x < m->nx; ++x) out[x] = 2.0 * lr[x] - po[x] + m->dt2 * lap_at(m, t, x);
  }
}

/* Mur edges of un from the same step, then the corners from the updated edges */
static void apply_mur(const Medium* m, const double* u, double* un) {
  const int ny = m->ny, nx = m->nx;
  for (int y = 1; y < ny - 1; ++y) {
    AT(m, un, y, 0) = mur1(m->kl[y], AT(m, u, y, 1), AT(m, un, y, 1), AT(m, u, y, 0));
    AT(m, un, y, nx - 1) = mur1(m->kr[y], AT(m, u, y, nx - 2), AT(m, un, y, nx - 2), AT(m, u, y, nx - 1));
  }
  for (int x = 1; x < nx - 1; ++x) {
    AT(m, un, 0, x) = mur1(m->kb[x], AT(m, u, 1, x), AT(m, un, 1, x), AT(m, u, 0, x));
    AT(m, un, ny - 1, x) = mur1(m->kt[x], AT(m, u, ny - 2, x), AT(m, un, ny - 2, x), AT(m, u, ny - 1, x));
  }
  double v[4];
  for (int q = 0; q < 4; ++q) {
    const double cu = AT(m, u, m->cy[q], m->cx[q]);
    const double fx = mur1(m->kcx[q], AT(m, u, m->cy[q], m->ix[q]), AT(m, un, m->cy[q], m->ix[q]), cu);
    const double fy = mur1(m->kcy[q], AT(m, u, m->iy[q], m->cx[q]), AT(m, un, m->iy[q], m->cx[q]), cu);
    v[q] = 0.5 * (fx + fy);
  }
  for (int q = 0; q < 4; ++q) AT(m, un, m->cy[q], m->cx[q]) = v[q];
}

typedef struct {
  int n_src; const int* row; const int* col; const double* w; const double* wave; int wave_len;
  int n_rx; const int* row0; const int* col0; const double* rw;
} Acq;

static void inject(const Medium* m, const Acq* a, double* un, int step) {
  if (step >= a->wave_len) return;
  const double v = a->wave[step];
  for (int k = 0; k < a->n_src; ++k) AT(m, un, a->row[k], a->col[k]) += a->w[k] * v;
}

static void record(const Medium* m, const Acq* a, const double* un, double* traces, int n_steps, int step) {
  for (int r = 0; r < a->n_rx; ++r) {
    const double* f = &AT(m, un, a->row0[r], a->col0[r]);
    const double* w = a->rw + 4 * (size_t)r;
    traces[(size_t)r * n_steps + step] = f[0] * w[0] + f[1] * w[1] + f[m->W] * w[2] + f[m->W + 1] * w[3];
  }
}

static int medium_setup(Medium* m, int ny, int nx, double dx, double dy, double dt, const double* c, int pml,
                        double pml_r) {
  if (medium_init(m, ny, nx, dx, dy, dt, c)) return 2;
  if (pml > 0 && medium_pml(m, c, dx, dy, dt, pml, pml_r)) { medium_free(m); return 2; }
  return 0;
}

/* One forward step (u-, u) -> un with sources and the edges (Mur, or the PML's
   face fields ps -> psn) */
static void forward_step(const Medium* m, const Acq* a, const double* uo, const double* u, double* un,
                         const double* psx, const double* psy, double* psxn, double* psyn, int step) {
  if (m->pml) {
    step_pml(m, uo, u, un, psx, psy, psxn, psyn);
    inject(m, a, un, step);
  } else {
    step_forward(m, uo, u, un);
    inject(m, a, un, step);
    apply_mur(m, u, un);
  }
}

/* Shot of a padded grid when pml > 0: the medium, sources and receivers are
   given on the padded grid (the layer included); pml_r is the target
   reflection of the damping profile. */
int orc_forward_shot(int ny, int nx, double dx, double dy, double dt, const double* c,
                     int n_src, const int* s_row, const int* s_col, const double* s_w,
                     const double* wave, int wave_len, int n_rx, const int* r_row0,
                     const int* r_col0, const double* r_w, int n_steps, double* traces, int pml,
                     double pml_r) {
  if (ny < 3 || nx < 3 || n_steps < 1) return 1;
  Medium m;
  if (medium_setup(&m, ny, nx, dx, dy, dt, c, pml, pml_r)) return 2;
  const Acq a = {n_src, s_row, s_col, s_w, wave, wave_len, n_rx, r_row0, r_col0, r_w};
  double* buf = (double*)calloc(7 * m.n, sizeof(double));
  if (!buf) { medium_free(&m); return 2; }
  double* uo = buf;
  double* u = buf + m.n;
  double* un = buf + 2 * m.n;
  double* ps[2][2] = {{buf + 3 * m.n, buf + 4 * m.n}, {buf + 5 * m.n, buf + 6 * m.n}};
  for (int step = 0; step < n_steps; ++step) {
    const int cur = step & 1;
    forward_step(&m, &a, uo, u, un, ps[cur][0], ps[cur][1], ps[cur ^ 1][0], ps[cur ^ 1][1], step);
    record(&m, &a, un, traces, n_steps, step);
    double* t = uo; uo = u; u = un; un = t;
  }
  free(buf);
  medium_free(&m);
  return 0;
}

/* Misfit 0.5 sum(r^2) and g_{c^2} (added into g, (ny, nx)) of one shot, with
   residual r = traces - observed and receiver channel `mute` zeroed (mute < 0:
   none): the forward keeps (u-, u) every ckpt_every steps, and the reverse sweep
   recomputes each segment before running the adjoint over it. */
int orc_gradient_shot(int ny, int nx, double dx, double dy, double dt, const double* c,
                      int n_src, const int* s_row, const int* s_col, const double* s_w,
                      const double* wave, int wave_len, int n_rx, const int* r_row0,
                      const int* r_col0, const double* r_w, int n_steps, const double* observed,
                      int mute, int ckpt_every, double* misfit, double* g, int pml, double pml_r) {
  if (ny < 3 || nx < 3 || n_steps < 1 || ckpt_every < 1) return 1;
  Medium m;
  if (medium_setup(&m, ny, nx, dx, dy, dt, c, pml, pml_r)) return 2;
  const Acq a = {n_src, s_row, s_col, s_w, wave, wave_len, n_rx, r_row0, r_col0, r_w};
  const int C = ckpt_every, nseg = (n_steps + C - 1) / C;
  const int NF = 4;  /* a checkpoint: u-, u and the two face fields */
  double* res = (double*)malloc(sizeof(double) * (size_t)n_rx * n_steps);
  double* ck = (double*)calloc((size_t)nseg * NF * m.n, sizeof(double));
  double* hist = (double*)calloc((size_t)(C + 1) * m.n, sizeof(double));
  double* work = (double*)calloc(15 * m.n, sizeof(double));
  if (!res || !ck || !hist || !work) { free(res); free(ck); free(hist); free(work); medium_free(&m); return 2; }
  double *uo = work, *u = work + m.n, *un = work + 2 * m.n;
  double* ps[2][2] = {{work + 7 * m.n, work + 8 * m.n}, {work + 9 * m.n, work + 10 * m.n}};
  double* qs[2][2] = {{work + 11 * m.n, work + 12 * m.n}, {work + 13 * m.n, work + 14 * m.n}};
  /* forward, keeping the state before steps 0, C, 2C, ... */
  int cur = 0;
  for (int step = 0; step < n_steps; ++step) {
    if (step % C == 0) {
      double* dst = ck + (size_t)(step / C) * NF * m.n;
      memcpy(dst, uo, m.n * sizeof(double));
      memcpy(dst + m.n, u, m.n * sizeof(double));
      memcpy(dst + 2 * m.n, ps[cur][0], m.n * sizeof(double));
      memcpy(dst + 3 * m.n, ps[cur][1], m.n * sizeof(double));
    }
    forward_step(&m, &a, uo, u, un, ps[cur][0], ps[cur][1], ps[cur ^ 1][0], ps[cur ^ 1][1], step);
    cur ^= 1;
    record(&m, &a, un, res, n_steps, step);
    double* t = uo; uo = u; u = un; un = t;
  }
  double J = 0.0;
  for (int r = 0; r < n_rx; ++r)
    for (int k = 0; k < n_steps; ++k) {
      const size_t i = (size_t)r * n_steps + k;
      const double v = (r == mute) ? 0.0 : res[i] - observed[i];
      res[i] = v;
      J += v * v;
    }
  *misfit = 0.5 * J;
  /* reverse sweep */
  double *lo = work + 3 * m.n, *l = work + 4 * m.n, *ln = work + 5 * m.n, *tmp = work + 6 * m.n;
  memset(lo, 0, 4 * m.n * sizeof(double));
  double* src = (double*)calloc(m.n, sizeof(double));
  if (!src) { free(res); free(ck); free(hist); free(work); medium_free(&m); return 2; }
  int qc = 0;  /* the adjoint's face fields (PML) */
  for (int j = nseg - 1; j >= 0; --j) {
    const int k0 = j * C, k1 = (k0 + C < n_steps) ? k0 + C : n_steps;
    const double* src_ck = ck + (size_t)j * NF * m.n;
    memcpy(uo, src_ck, m.n * sizeof(double));
    memcpy(u, src_ck + m.n, m.n * sizeof(double));
    cur = 0;
    memcpy(ps[0][0], src_ck + 2 * m.n, m.n * sizeof(double));
    memcpy(ps[0][1], src_ck + 3 * m.n, m.n * sizeof(double));
    memcpy(hist, u, m.n * sizeof(double));              /* u after step k0 - 1 */
    for (int step = k0; step < k1; ++step) {
      forward_step(&m, &a, uo, u, un, ps[cur][0], ps[cur][1], ps[cur ^ 1][0], ps[cur ^ 1][1], step);
      cur ^= 1;
      memcpy(hist + (size_t)(step - k0 + 1) * m.n, un, m.n * sizeof(double));  /* u after step */
      double* t = uo; uo = u; u = un; un = t;
    }
    for (int n = k1 - 1; n >= k0; --n) {
      /* scatter of residual column n (the transpose of the bilinear gather), in the
         reference's index_put_ order: all w00 taps, then w10, w01, w11 */
      for (int tap = 0; tap < 4; ++tap)
        for (int r = 0; r < n_rx; ++r) {
          const int yy = r_row0[r] + (tap >= 2), xx = r_col0[r] + (tap & 1);
          AT(&m, src, yy, xx) += res[(size_t)r * n_steps + n] * r_w[4 * (size_t)r + tap];
        }
      if (m.pml) {
        /* PML grids carry the adjoint as w = (c dt)^2 l with the forward's PML step
           (the layer absorbs the adjoint wave as it does the forward one); the
           injection is scaled by (c dt)^2 */
        step_pml(&m, lo, l, ln, qs[qc][0], qs[qc][1], qs[qc ^ 1][0], qs[qc ^ 1][1]);
        qc ^= 1;
      } else {
        step_adjoint(&m, lo, l, ln, tmp);
      }
      for (int tap = 0; tap < 4; ++tap)
        for (int r = 0; r < n_rx; ++r) {
          const int yy = r_row0[r] + (tap >= 2), xx = r_col0[r] + (tap & 1);
          /* a node shared by several taps adds its sum once, then holds 0 */
          const double v = AT(&m, src, yy, xx);
          AT(&m, ln, yy, xx) += m.pml ? AT(&m, m.k2, yy, xx) * v : v;
          AT(&m, src, yy, xx) = 0.0;
        }
      if (!m.pml) apply_mur(&m, l, ln);
      double* t = lo; lo = l; l = ln; ln = t;
      if (n >= 1) {
        const double* w = hist + (size_t)(n - k0) * m.n;  /* u after step n - 1 */
        for (int y = 0; y < ny; ++y) {
          const double* wr = &AT(&m, w, y, 0);
          const double* lr = &AT(&m, l, y, 0);
          const double* kr = &AT(&m, m.k2, y, 0);
          double* gr = g + (size_t)y * nx;
          if (m.pml) {
            for (int x = 0; x < nx; ++x) gr[x] += m.dt2 * ((lr[x] / kr[x]) * lap_at(&m, wr, x));
          } else {
            for (int x = 0; x < nx; ++x) gr[x] += m.dt2 * (lr[x] * lap_at(&m, wr, x));
          }
        }
      }
    }
  }
  free(src);
  free(res);
  free(ck);
  free(hist);
  free(work);
  medium_free(&m);
  return 0;
}
