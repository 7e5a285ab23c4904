// One register-budget variant of the section-move kernel per translation unit
// (compiled with -DPIMC_NT=256 -DPIMC_MINB=2, 3, 4, and -DPIMC_NT=512
// -DPIMC_MINB=1; and for launches without node models -DPIMC_NODES=0 with
// MINB 2, 3, 4), so the variants build in parallel.
#include <cuda_runtime.h>

#include "kernels.cuh"

#ifndef PIMC_MINB
#error "compile with -DPIMC_MINB=<minimum resident blocks per SM>"
#endif
#ifndef PIMC_NT
#define PIMC_NT 256
#endif
// -DPIMC_NODES=0: the variant without the fixed-node phases (launches whose
// systems have no node models), its entry points named *_nf_v<MINB>
#ifndef PIMC_NODES
#define PIMC_NODES 1
#endif
#define PIMC_CAT2(a, b) a##b
#define PIMC_CAT(a, b) PIMC_CAT2(a, b)
#if PIMC_NODES
#define PIMC_NAME(base) PIMC_CAT(base##_v, PIMC_MINB)
#else
#define PIMC_NAME(base) PIMC_CAT(base##_nf_v, PIMC_MINB)
#endif
#define PIMC_KERNEL section_moves_kernel<PIMC_NT, PIMC_MINB, (PIMC_NODES != 0)>

namespace pimc {

cudaError_t PIMC_NAME(section_launch)(int grid, int block, size_t smem, cudaStream_t stream,
                                      const RunParams& P) {
  PIMC_KERNEL<<<grid, block, smem, stream>>>(P);
  return cudaGetLastError();
}

int PIMC_NAME(section_occupancy)(int block, size_t smem) {
  int occ = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, PIMC_KERNEL, block, smem) != cudaSuccess)
    return 0;
  return occ;
}

void PIMC_NAME(section_smem_cap)(int bytes) {
  cudaFuncSetAttribute(PIMC_KERNEL, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}

}  // namespace pimc
