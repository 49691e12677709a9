// Temporally blocked adjoint launches (imaging included) for grids with Mur edges:
// the kernel templates of fdtd_tb.cuh instantiated for the adjoint only, in a
// translation unit of their own so that the families compile in parallel.

#include "fdtd_tb.cuh"

namespace fdtd {

cudaError_t tb_launch_adj(const TbParams& p, int ky, int grid, size_t smem, cudaStream_t st) {
  return launch_shape<MODE_ADJ, false>(p, ky, grid, smem, st);
}

cudaError_t tb_configure_adj(int ky, int nwarps, size_t smem) {
  return configure_shape<MODE_ADJ, false>(ky, nwarps, smem);
}

cudaError_t tb_group_launch_adj(const TbGroup& g, int ky, int nwarps, bool adj_coef, int grid, size_t smem,
                                cudaStream_t st) {
  return group_shape<MODE_ADJ>(g, ky, nwarps, adj_coef, grid, smem, st);
}

}  // namespace fdtd
