// One register-budget variant of the section-move kernel per translation unit
// (compiled with -DPIMC_NT=256 -DPIMC_MINB=2, 3, 4, and -DPIMC_NT=512
// -DPIMC_MINB=1), so the variants build in parallel.
#include <cuda_runtime.h>

#include "kernels.cuh"

#ifndef PIMC_MINB
#error "compile with -DPIMC_MINB=<minimum resident blocks per SM>"
#endif
#ifndef PIMC_NT
#define PIMC_NT 256
#endif
#define PIMC_CAT2(a, b) a##b
#define PIMC_CAT(a, b) PIMC_CAT2(a, b)

namespace pimc {

cudaError_t PIMC_CAT(section_launch_v, PIMC_MINB)(int grid, int block, size_t smem,
                                                    cudaStream_t stream, const RunParams& P) {
  section_moves_kernel<PIMC_NT, PIMC_MINB><<<grid, block, smem, stream>>>(P);
  return cudaGetLastError();
}

int PIMC_CAT(section_occupancy_v, PIMC_MINB)(int block, size_t smem) {
  int occ = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, section_moves_kernel<PIMC_NT, PIMC_MINB>, block,
                                                    smem) != cudaSuccess)
    return 0;
  return occ;
}

void PIMC_CAT(section_smem_cap_v, PIMC_MINB)(int bytes) {
  cudaFuncSetAttribute(section_moves_kernel<PIMC_NT, PIMC_MINB>,
                       cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}

}  // namespace pimc
