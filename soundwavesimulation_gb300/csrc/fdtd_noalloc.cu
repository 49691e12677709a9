// fdtd_forward_plain_static: the plain per-shot forward with its scratch in a
// fixed device array, for callers that cannot allocate device memory.
//
// Some callers have no way to obtain device memory for a workspace: processes
// whose device memory is owned entirely by another allocator (a framework's
// caching pool or a fixed arena set up at start-up), and programs that bind the
// C ABI from an environment without a device allocator, which hold only their
// input/output buffers and a stream. This entry point serves them: it takes the
// same problem description and traces buffer as fdtd_forward_plain but no
// workspace, and it calls no cudaMalloc, cudaFree or allocating library routine.
// On success it does not touch the host heap either; only a failing call builds
// the message that fdtd_last_error() returns.
//
// The scratch is `g_plain_scratch` below: FDTD_STATIC_SCRATCH_BYTES of device
// memory that every GPU loading this library holds until the process exits. On
// its first call on a device (with that device current) the entry point looks up
// the array's device address once with cudaGetSymbolAddress and caches it; make
// that first call before any stream capture. The cached address belongs to the
// device's primary context: a cudaDeviceReset, or a caller that runs in another
// context of the same device, is not supported. Every call copies the receiver
// and source tables from the caller's host arrays into the array and then
// synchronises `stream` before it launches the time loop. All calls share the
// array and it keeps the last call's contents, so every field it uses is cleared
// at the start of each shot; calls that overlap on the GPU (other streams, other
// threads) race on the array.

#include <mutex>

#include "../../include/fdtd_gb300.h"
#include "fdtd_internal.h"

namespace fdtd {
namespace {

__device__ __align__(256) unsigned char g_plain_scratch[FDTD_STATIC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
void* g_scratch_addr[kMaxDevices] = {};
std::mutex g_scratch_mutex;

size_t round256(size_t v) { return (v + 255) / 256 * 256; }

}  // namespace
}  // namespace fdtd

using namespace fdtd;

extern "C" int32_t fdtd_forward_plain_static(const fdtd_problem* prob, float* traces, void* stream) {
  if (!prob || !traces) return fail(FDTD_ERR_INVALID, "null argument");
  // the same checks as fdtd_forward_plain: grid, spacings, receivers and every
  // used source entry (node inside the grid, waveform index below n_waves)
  const int32_t bad = validate_plain_problem(*prob);
  if (bad) return bad;
  const fdtd_grid& g = prob->grid;
  const int R = prob->rx.n, S = prob->n_shots, nt = prob->n_steps;
  const int K = prob->src.per_shot;
  const size_t plane = (size_t)g.ny * g.pitch;
  const size_t off_rc = round256(3 * plane * sizeof(float));
  const size_t off_w = off_rc + round256((size_t)R * 2 * sizeof(int32_t));
  const size_t off_src = off_w + round256((size_t)R * 4 * sizeof(float));
  const size_t need = off_src + round256((size_t)S * K * 4 * sizeof(int32_t));
  if (need > (size_t)FDTD_STATIC_SCRATCH_BYTES) {
    return fail(FDTD_ERR_WORKSPACE,
                "fdtd_forward_plain_static: problem needs " + std::to_string(need) +
                " bytes of scratch, more than the fixed " + std::to_string((size_t)FDTD_STATIC_SCRATCH_BYTES) +
                " bytes (3 fields of one shot plus tables); use fdtd_forward_plain with a workspace");
  }
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  if (dev < 0 || dev >= kMaxDevices) return fail(FDTD_ERR_UNSUPPORTED, "device index out of range");
  void* base = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (!g_scratch_addr[dev]) {
      void* addr = nullptr;
      e = cudaGetSymbolAddress(&addr, g_plain_scratch);
      if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress of the static scratch");
      g_scratch_addr[dev] = addr;
    }
    base = g_scratch_addr[dev];
  }
  cudaStream_t st = (cudaStream_t)stream;
  char* w = reinterpret_cast<char*>(base);
  float* f[3] = {reinterpret_cast<float*>(w), reinterpret_cast<float*>(w) + plane,
                 reinterpret_cast<float*>(w) + 2 * plane};
  int32_t* rx_rc = reinterpret_cast<int32_t*>(w + off_rc);
  float* rx_w = reinterpret_cast<float*>(w + off_w);
  int32_t* s_row = reinterpret_cast<int32_t*>(w + off_src);
  int32_t* s_col = s_row + (size_t)S * K;
  int32_t* s_wave = s_col + (size_t)S * K;
  float* s_w = reinterpret_cast<float*>(s_wave + (size_t)S * K);
  // receiver (row0, col0) pairs interleaved by two strided copies, no host buffer
  e = cudaMemcpy2DAsync(rx_rc, 2 * sizeof(int32_t), prob->rx.row0, sizeof(int32_t), sizeof(int32_t), R,
                        cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess)
    e = cudaMemcpy2DAsync(rx_rc + 1, 2 * sizeof(int32_t), prob->rx.col0, sizeof(int32_t), sizeof(int32_t), R,
                          cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(rx_w, prob->rx.w, (size_t)R * 16, cudaMemcpyHostToDevice, st);
  if (K > 0) {
    const size_t n = (size_t)S * K * 4;
    if (e == cudaSuccess) e = cudaMemcpyAsync(s_row, prob->src.row, n, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(s_col, prob->src.col, n, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(s_wave, prob->src.wave, n, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(s_w, prob->src.w, n, cudaMemcpyHostToDevice, st);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(e, "static forward upload");
  for (int s = 0; s < S; ++s) {
    e = cudaMemsetAsync(w, 0, 3 * plane * sizeof(float), st);  // the array keeps the last call's fields
    if (e != cudaSuccess) return cuda_fail(e, "static forward reset");
    int io = 0, ic = 1, in = 2;
    for (int n = 0; n < nt; ++n) {
      int32_t rc = fdtd_step(&g, 1, f[io], f[ic], f[in], K, s_row + (size_t)s * K, s_col + (size_t)s * K,
                             s_w + (size_t)s * K, s_wave + (size_t)s * K, prob->src.waveforms,
                             prob->src.waveform_len, n, nullptr, 0, stream);
      if (rc) return rc;
      e = gather_launch(g.ny, g.pitch, 1, f[in], R, rx_rc, rx_w, traces + (size_t)s * R * nt + n, 0, nt, st);
      if (e != cudaSuccess) return cuda_fail(e, "static forward gather");
      const int t = io; io = ic; ic = in; in = t;
    }
  }
  return FDTD_OK;
}
