// The allocation-free node-evaluation kernel and its static scratch (one
// translation unit only: the scratch is a __device__ array).
#pragma once
#include "entry_kernels.cuh"

namespace pimc {

// ------------------------------------------- allocation-free node evaluation
// Scratch for node_eval_noalloc_kernel: one slot of 6 * 32 * 32 + 33 doubles
// (rounded up to 6208: the LU, inverse and exp matrices, pivot reciprocals and
// the three gradient matrices of free-particle nodes, for one Slater matrix of
// up to 32 particles) per resident warp, kNoAllocSlots slots: 6.1 MiB, held by
// every GPU that loads the library until exit.
constexpr int kNoAllocSlots = 128;
constexpr int kNoAllocSlot = (node_group_scratch(kMaxNs) + 31) / 32 * 32;
__device__ __align__(256) double g_noalloc_scratch[kNoAllocSlots * kNoAllocSlot];

struct NoAllocParams {
  DevSys sys;  // by value: nothing to allocate
  const double* r1;
  const double* r2;
  double* det;
  double* d1;
  double* d2;
  int* err;
  double scale;
  int ispec;
  int nbatch;
  double* scratch;  // device address of g_noalloc_scratch
};

// One warp per block; block b takes batch entries b, b + gridDim.x, ... and
// uses scratch slot b.  Positions are staged in dynamic shared memory
// (6 * npart doubles), which is part of the launch, not an allocation.
__global__ void __launch_bounds__(32) node_eval_noalloc_kernel(NoAllocParams P) {
  extern __shared__ double sh[];
  const DevSys& s = P.sys;
  const int np = s.npart, sp = P.ispec;
  double* sx = sh;
  double* sy = sx + 2 * np;
  double* sz = sy + 2 * np;
  double* scr = P.scratch + (size_t)blockIdx.x * kNoAllocSlot;
  const int f = s.spec_first[sp];
  for (int b = blockIdx.x; b < P.nbatch; b += gridDim.x) {
    for (int i = threadIdx.x; i < np; i += 32) {
      sx[i] = P.r1[((size_t)b * np + i) * 3];
      sy[i] = P.r1[((size_t)b * np + i) * 3 + 1];
      sz[i] = P.r1[((size_t)b * np + i) * 3 + 2];
      sx[np + i] = P.r2[((size_t)b * np + i) * 3];
      sy[np + i] = P.r2[((size_t)b * np + i) * 3 + 1];
      sz[np + i] = P.r2[((size_t)b * np + i) * 3 + 2];
      P.d1[(size_t)b * np + i] = 200;
      P.d2[(size_t)b * np + i] = 200;
    }
    __syncwarp();
    SliceView v1{sx, sy, sz, np, 0, -1, 0, 0, 0};
    SliceView v2{sx, sy, sz, np, 1, -1, 0, 0, 0};
    double det;
    int err;
    node_eval_warp(s, sp, v1, v2, P.scale, scr, 1, det, err, P.d1 + (size_t)b * np + f,
                   P.d2 + (size_t)b * np + f);
    if (threadIdx.x == 0) {
      P.det[b] = det;
      P.err[b] = err;
    }
    __syncwarp();
  }
}

}  // namespace pimc
