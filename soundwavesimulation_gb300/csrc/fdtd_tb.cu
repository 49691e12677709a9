// Temporally blocked kernel launches for grids with Mur edges: the forward (also the
// form that keeps the stencil stream) and the recompute here, the adjoint in
// fdtd_tb_adj.cu and the PML family in
// fdtd_tb_pml.cu / fdtd_tb_pml_adj.cu (the kernel templates are in fdtd_tb.cuh).
// Each translation unit compiles its own instantiations, in parallel.

#include "fdtd_tb.cuh"

namespace fdtd {

cudaError_t tb_launch(const TbParams& p, int ky, int mode, int grid, size_t smem, cudaStream_t st) {
  if (mode == MODE_FWDQ) {  // grids without PML only
    if (p.pml) return cudaErrorInvalidValue;
    return launch_shape<MODE_FWDQ, false>(p, ky, grid, smem, st);
  }
  if (p.pml) return tb_launch_pml(p, ky, mode, grid, smem, st);
  if (mode == MODE_FWD) return launch_shape<MODE_FWD, false>(p, ky, grid, smem, st);
  if (mode == MODE_REC) return launch_shape<MODE_REC, false>(p, ky, grid, smem, st);
  return tb_launch_adj(p, ky, grid, smem, st);
}

cudaError_t tb_group_launch(const TbGroup& g, int ky, int nwarps, int mode, bool adj_coef, int grid, size_t smem,
                            cudaStream_t st) {
  if (mode == MODE_FWD) return group_shape<MODE_FWD>(g, ky, nwarps, adj_coef, grid, smem, st);
  if (mode == MODE_FWDQ) return group_shape<MODE_FWDQ>(g, ky, nwarps, adj_coef, grid, smem, st);
  if (mode == MODE_REC) return group_shape<MODE_REC>(g, ky, nwarps, adj_coef, grid, smem, st);
  return tb_group_launch_adj(g, ky, nwarps, adj_coef, grid, smem, st);
}

size_t tb_group_static_smem() { return sizeof(TbParams) + 16; }

cudaError_t tb_configure(int ky, int mode, int nwarps, size_t smem, bool pml) {
  if (smem + TB_STATIC_SMEM > 232448) return cudaSuccess;  // a mode this plan never launches
  if (mode == MODE_FWDQ) return pml ? cudaErrorInvalidValue : configure_shape<MODE_FWDQ, false>(ky, nwarps, smem);
  if (pml) return tb_configure_pml(ky, mode, nwarps, smem);
  if (mode == MODE_FWD) return configure_shape<MODE_FWD, false>(ky, nwarps, smem);
  if (mode == MODE_REC) return configure_shape<MODE_REC, false>(ky, nwarps, smem);
  return tb_configure_adj(ky, nwarps, smem);
}

}  // namespace fdtd
