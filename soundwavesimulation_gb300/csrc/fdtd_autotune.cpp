// fdtd_autotune: launch-shape search of the temporally blocked engine.
//
// For one acquisition, every candidate (rows per lane, warps, steps per launch)
// that the planner accepts for the grid is bound to the caller's workspace and
// timed with CUDA events on the caller's stream over `launches` temporal blocks
// (a forward, or with for_gradient a forward with checkpoints plus the adjoint),
// after one untimed pass; the fastest shape wins. The search allocates no device
// memory: the caller passes one workspace of fdtd_autotune_workspace_bytes().
// The reference has no tuner; its batch sizes come from auto_batch_size
// (fdtd2d/torch_backend.py:773-789) and its step is a fixed torch.compile graph.

#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "../../include/fdtd_gb300.h"
#include "fdtd_internal.h"

namespace {

constexpr size_t kAlign = 256;
size_t round_up(size_t v) { return (v + kAlign - 1) / kAlign * kAlign; }

const int kShapes[][2] = {{8, 16}, {8, 12}, {8, 10}, {4, 32}, {4, 16}};  // (rows per lane, warps)
const int kDepths[] = {6, 8, 10, 12, 15, 19, 23};                        // steps per launch

struct Probe {
  fdtd_tuning tuning;
  fdtd_problem problem;
  size_t plan_bytes;
};

// The probe problem of a candidate: the acquisition cut to `launches` blocks.
bool make_probe(const fdtd_problem& prob, int ky, int warps, int depth, int launches, int for_gradient, Probe& out) {
  std::memset(&out.tuning, 0, sizeof(out.tuning));
  out.tuning.rows_per_lane = ky;
  out.tuning.warps = warps;
  out.tuning.steps_per_launch = depth;
  out.problem = prob;
  out.problem.n_steps = std::min(prob.n_steps, std::max(1, launches) * depth);
  fdtd_plan* plan = nullptr;
  if (fdtd_plan_create(&out.problem, &out.tuning, for_gradient, &plan) != FDTD_OK) return false;
  fdtd_plan_workspace_bytes(plan, &out.plan_bytes);
  fdtd_plan_destroy(plan);
  return true;
}

size_t probe_bytes(const Probe& pr) {
  const fdtd_problem& q = pr.problem;
  const size_t traces = (size_t)q.n_shots * q.rx.n * q.n_steps * sizeof(float);
  const size_t grad = (size_t)q.grid.ny * q.grid.pitch * sizeof(double);
  return round_up(pr.plan_bytes) + round_up(traces) + round_up(grad);
}

}  // namespace

using namespace fdtd;

extern "C" {

size_t fdtd_autotune_workspace_bytes(const fdtd_problem* problem, int32_t for_gradient, int32_t launches) {
  if (!problem) return 0;
  size_t need = 0;
  for (const auto& sh : kShapes)
    for (int depth : kDepths) {
      Probe pr;
      if (make_probe(*problem, sh[0], sh[1], depth, launches, for_gradient, pr)) need = std::max(need, probe_bytes(pr));
    }
  return need;
}

int32_t fdtd_autotune(const fdtd_problem* problem, int32_t for_gradient, int32_t launches, int32_t repeats,
                      void* workspace, size_t bytes, fdtd_tuning* best, double* best_rate, fdtd_tuning* tried,
                      double* rates, int32_t* n_tried, void* stream) {
  if (!problem || !best) return fail(FDTD_ERR_INVALID, "null argument");
  if (!workspace) return fail(FDTD_ERR_WORKSPACE, "autotune workspace missing");
  if (launches < 1 || repeats < 1) return fail(FDTD_ERR_INVALID, "launches and repeats must be positive");
  cudaStream_t st = (cudaStream_t)stream;
  const int cap = n_tried ? *n_tried : 0;
  int count = 0;
  double top = 0.0;
  bool found = false;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaError_t e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  if (e != cudaSuccess) return cuda_fail(e, "autotune events");
  int32_t rc = FDTD_OK;
  for (const auto& sh : kShapes) {
    for (int depth : kDepths) {
      Probe pr;
      if (!make_probe(*problem, sh[0], sh[1], depth, launches, for_gradient, pr)) continue;  // shape does not fit
      if (probe_bytes(pr) > bytes) { rc = fail(FDTD_ERR_WORKSPACE, "autotune workspace too small"); goto done; }
      fdtd_plan* plan = nullptr;
      rc = fdtd_plan_create(&pr.problem, &pr.tuning, for_gradient, &plan);
      if (rc) goto done;
      char* ws = reinterpret_cast<char*>(workspace);
      float* traces = reinterpret_cast<float*>(ws + round_up(pr.plan_bytes));
      double* grad = reinterpret_cast<double*>(
          ws + round_up(pr.plan_bytes) +
          round_up((size_t)pr.problem.n_shots * pr.problem.rx.n * pr.problem.n_steps * sizeof(float)));
      float ms = 0.f;
      rc = fdtd_plan_bind(plan, ws, pr.plan_bytes, stream);
      // one untimed pass, then `repeats` timed ones; any residual serves the
      // adjoint (its cost does not depend on the values), so the traces do
      for (int k = 0; k <= repeats && rc == FDTD_OK; ++k) {
        if (k == 1 && (e = cudaEventRecord(e0, st)) != cudaSuccess) { rc = cuda_fail(e, "autotune event"); break; }
        rc = fdtd_forward(plan, traces, nullptr, nullptr, for_gradient, stream);
        if (rc == FDTD_OK && for_gradient) rc = fdtd_adjoint(plan, traces, grad, stream);
      }
      if (rc == FDTD_OK) {
        e = cudaEventRecord(e1, st);
        if (e == cudaSuccess) e = cudaEventSynchronize(e1);
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
        if (e != cudaSuccess) rc = cuda_fail(e, "autotune timing");
      }
      fdtd_plan_destroy(plan);
      if (rc) goto done;
      const double cells = (double)pr.problem.grid.ny * pr.problem.grid.nx * pr.problem.n_shots * pr.problem.n_steps;
      const double rate = cells * repeats / (ms * 1e-3) / 1e9;
      if (count < cap) {
        if (tried) tried[count] = pr.tuning;
        if (rates) rates[count] = rate;
      }
      ++count;
      if (!found || rate > top) {
        top = rate;
        *best = pr.tuning;
        found = true;
      }
    }
  }
  if (!found) rc = fail(FDTD_ERR_UNSUPPORTED, "no candidate launch shape fits this problem");
done:
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (n_tried) *n_tried = std::min(count, cap);
  if (rc == FDTD_OK && best_rate) *best_rate = top;
  return rc;
}

}  // extern "C"
