// Temporally blocked kernel launches for grids with Mur edges (the PML family is in
// fdtd_tb_pml.cu); the kernel templates are in fdtd_tb.cuh.

#include "fdtd_tb.cuh"

namespace fdtd {

cudaError_t tb_launch_pml(const TbParams& p, int ky, int mode, int grid, size_t smem, cudaStream_t st);
cudaError_t tb_configure_pml(int ky, int mode, int nwarps, size_t smem);

cudaError_t tb_launch(const TbParams& p, int ky, int mode, int grid, size_t smem, cudaStream_t st) {
  if (p.pml) return tb_launch_pml(p, ky, mode, grid, smem, st);
  return launch_shape<false>(p, ky, mode, grid, smem, st);
}

template <int KY, int MODE, int MAXT>
cudaError_t group_one(const TbGroup& g, int nwarps, int grid, size_t smem, cudaStream_t st) {
  static size_t configured_smem = 0;
  if (smem > configured_smem) {
    cudaError_t e = cudaFuncSetAttribute(tb_group_kernel<KY, MODE, MAXT>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    configured_smem = smem;
  }
  tb_group_kernel<KY, MODE, MAXT><<<grid, nwarps * 32, smem, st>>>(g);
  return cudaGetLastError();
}

template <int KY, int MAXT>
cudaError_t group_mode(const TbGroup& g, int nwarps, int mode, int grid, size_t smem, cudaStream_t st) {
  if (mode == MODE_FWD) return group_one<KY, MODE_FWD, MAXT>(g, nwarps, grid, smem, st);
  if (mode == MODE_REC) return group_one<KY, MODE_REC, MAXT>(g, nwarps, grid, smem, st);
  return group_one<KY, MODE_ADJ, MAXT>(g, nwarps, grid, smem, st);
}

cudaError_t tb_group_launch(const TbGroup& g, int ky, int nwarps, int mode, int grid, size_t smem,
                            cudaStream_t st) {
  if (ky == 8) {
    if (nwarps <= 12) return group_mode<8, 384>(g, nwarps, mode, grid, smem, st);
    return group_mode<8, 512>(g, nwarps, mode, grid, smem, st);
  }
  if (nwarps <= 16) return group_mode<4, 512>(g, nwarps, mode, grid, smem, st);
  return group_mode<4, 1024>(g, nwarps, mode, grid, smem, st);
}

size_t tb_group_static_smem() { return sizeof(TbParams) + 16; }

cudaError_t tb_configure(int ky, int mode, int nwarps, size_t smem, bool pml) {
  if (smem > 232448) return cudaSuccess;  // a mode this plan never launches
  if (pml) return tb_configure_pml(ky, mode, nwarps, smem);
  return configure_shape<false>(ky, mode, nwarps, smem);
}

}  // namespace fdtd
