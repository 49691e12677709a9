// Temporally blocked kernel launches for grids with a PML layer: the same kernel
// templates (fdtd_tb.cuh) instantiated with the PML step, in a translation unit of
// their own so that the Mur family keeps its register allocation.

#include "fdtd_tb.cuh"

namespace fdtd {

cudaError_t tb_launch_pml(const TbParams& p, int ky, int mode, int grid, size_t smem, cudaStream_t st) {
  return launch_shape<true>(p, ky, mode, grid, smem, st);
}

cudaError_t tb_configure_pml(int ky, int mode, int nwarps, size_t smem) {
  return configure_shape<true>(ky, mode, nwarps, smem);
}

}  // namespace fdtd
