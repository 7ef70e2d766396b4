// The FP32 single-CTA solve kernel whose layouts hold the steepest-edge
// column norms as partial sums of every row group, with the norm region
// grown to fit them (solve_kernel<float, false, true>).  The plan code in
// blpg_api.cu picks it for a class only where that growth costs no CTAs per
// SM; it lives in its own translation unit so that it compiles beside the
// other kernels instead of after them.
#include <cuda_runtime.h>

#include "blpg_internal.h"
#include "blpg_solver.cuh"

namespace blpg {

cudaError_t part_set_attrs(int max_smem) {
  return cudaFuncSetAttribute(dev::solve_kernel<float, false, true>,
                              cudaFuncAttributeMaxDynamicSharedMemorySize, max_smem);
}

cudaError_t part_occupancy(int* ctas_per_sm, int nt, int smem) {
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(
      ctas_per_sm, dev::solve_kernel<float, false, true>, nt, smem);
}

cudaError_t part_launch(int grid, int nt, int smem, cudaStream_t s, const dev::LpArgs& a,
                        const dev::ClassArgs& ca) {
  dev::solve_kernel<float, false, true><<<grid, nt, smem, s>>>(a, ca);
  return cudaGetLastError();
}

}  // namespace blpg
