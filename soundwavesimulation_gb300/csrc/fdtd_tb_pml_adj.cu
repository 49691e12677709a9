// Temporally blocked adjoint launches for grids with a PML layer (the kernel
// templates of fdtd_tb.cuh with the PML step), in a translation unit of their own.

#include "fdtd_tb.cuh"

namespace fdtd {

cudaError_t tb_launch_pml_adj(const TbParams& p, int ky, int grid, size_t smem, cudaStream_t st) {
  return launch_shape<MODE_ADJ, true>(p, ky, grid, smem, st);
}

cudaError_t tb_configure_pml_adj(int ky, int nwarps, size_t smem) {
  return configure_shape<MODE_ADJ, true>(ky, nwarps, smem);
}

}  // namespace fdtd
