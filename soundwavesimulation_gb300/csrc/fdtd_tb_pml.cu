// Temporally blocked kernel launches for grids with a PML layer: the same kernel
// templates (fdtd_tb.cuh) instantiated with the PML step, in translation units of
// their own (the forward and recompute here, the adjoint in fdtd_tb_pml_adj.cu) so
// that the Mur family keeps its register allocation and the units compile in
// parallel.

#include "fdtd_tb.cuh"

namespace fdtd {

cudaError_t tb_launch_pml(const TbParams& p, int ky, int mode, int grid, size_t smem, cudaStream_t st) {
  if (mode == MODE_FWD) return launch_shape<MODE_FWD, true>(p, ky, grid, smem, st);
  if (mode == MODE_REC) return launch_shape<MODE_REC, true>(p, ky, grid, smem, st);
  return tb_launch_pml_adj(p, ky, grid, smem, st);
}

cudaError_t tb_configure_pml(int ky, int mode, int nwarps, size_t smem) {
  if (mode == MODE_FWD) return configure_shape<MODE_FWD, true>(ky, nwarps, smem);
  if (mode == MODE_REC) return configure_shape<MODE_REC, true>(ky, nwarps, smem);
  return tb_configure_pml_adj(ky, nwarps, smem);
}

}  // namespace fdtd
