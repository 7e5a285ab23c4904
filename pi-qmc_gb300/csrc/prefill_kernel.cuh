// Filling the path-resident Slater-result cache in parallel: every (replica,
// node species, slice pair (t, t + M/2)) entry evaluated by its own warp, with
// exactly the arithmetic node_initialize uses on a miss (NodeModel::evaluate +
// evaluateDistance at the replica's current scale), so an entry filled here is
// the entry the section kernel would have filled.  This takes a replica's
// first visits of its slices off the section kernel's sequential path (a
// freshly uploaded path, a newly admitted request).
#pragma once
#include "kernels.cuh"

namespace pimc {

// Newly arrived paths are scanned for non-finite coordinates: a replica holding
// one gets PIMC_STATUS_NONFINITE at upload, before any move reads the bead
// (pi-qmc has no such check; a NaN would propagate through its actions
// silently).  Block (x, y) scans a 1/gridDim.x share of the paths of replicas
// y, y + gridDim.y, ...  The replica's moves still run: every table index and
// lane choice in the kernels stays in bounds for non-finite inputs (float to
// int conversions of NaN give 0, pivot searches pick among the group's own
// lanes), so the status word is the whole effect on the other replicas.
__global__ void __launch_bounds__(kBlock) path_scan_kernel(const DevSys* sys, DevState* state,
                                                           const double* paths, int nrep) {
  for (int r = blockIdx.y; r < nrep; r += gridDim.y) {
    const long long n = 3LL * sys[r].nslice * sys[r].npart;
    const double* p = paths + sys[r].path_offset;
    int bad = 0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
      bad |= !isfinite(p[i]);
    if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(&state[r].status, (uint32_t)PIMC_STATUS_NONFINITE);
  }
}

// An upload of paths over the engine's current ones (pimc_upload_paths):
// block (t, r) compares slice t of replica r bit for bit, copies it when it
// differs and flags it in changed[r][t] (nslice_max per replica).
__global__ void __launch_bounds__(kBlock) path_update_kernel(const DevSys* sys, double* paths,
                                                             const double* upload,
                                                             unsigned char* changed,
                                                             int nslice_max, int nrep) {
  const int t = blockIdx.x;
  for (int r = blockIdx.y; r < nrep; r += gridDim.y) {  // block-uniform
    const DevSys& s = sys[r];
    if (t >= s.nslice) continue;
    const int n = 3 * s.npart;
    const size_t o = s.path_offset + (size_t)t * n;
    const long long* a = (const long long*)(paths + o);
    const long long* b = (const long long*)(upload + o);
    int diff = 0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) diff |= a[i] != b[i];
    diff = __syncthreads_or(diff);
    if (diff)
      for (int i = threadIdx.x; i < n; i += blockDim.x) paths[o + i] = upload[o + i];
    if (threadIdx.x == 0) changed[(size_t)r * nslice_max + t] = diff ? 1 : 0;
  }
}

// The Slater-result entries that pair a changed slice (as r1 on slice t or as
// r2 on slice t - M/2) are invalidated: entry (r, species, t) for a changed t
// or t + M/2.
__global__ void cache_invalidate_kernel(const DevSys* sys, double* cache,
                                        const unsigned char* changed, int nslice_max, int nrep) {
  const double NaN = __longlong_as_double(0x7ff8000000000000LL);
  for (int r = blockIdx.y; r < nrep; r += gridDim.y) {
    const DevSys& s = sys[r];
    if (!s.fixed_node || s.nc_offset < 0) continue;
    const int M = s.nslice;
    const unsigned char* c = changed + (size_t)r * nslice_max;
    for (int it = blockIdx.x * blockDim.x + threadIdx.x; it < s.nspecies * M;
         it += gridDim.x * blockDim.x) {
      const int sp = it / M, t = it - sp * M;
      if (!s.node_kind[sp]) continue;
      if (c[t] || c[(t + M / 2) % M])
        cache[s.nc_offset + ((size_t)sp * M + t) * s.nc_stride] = NaN;
    }
  }
}

struct PrefillParams {
  const DevSys* sys;
  const DevState* state;
  const double* paths;
  double* cache;       // the cache pool (entries at sys.nc_offset)
  const int* slots;    // replicas to fill (null: 0 .. nslot-1)
  int nslot;
  int only_invalid;    // skip the entries that are valid (of the current scale)
  int ntask_per_slot;  // nspecies_max x nslice_max
  int stage_stride;    // doubles of slice-pair staging per warp (6 n_max)
  int scratch_stride;  // doubles of Slater scratch per warp (its hot part when split)
  double* gscratch;    // per-warp Slater scratch in global memory (null: shared memory)
  double* gcold;       // per-warp cold parts in global memory when split (null: not split)
  int cold_stride;     // doubles of cold part per warp
};

// Warps loop over the (slot, species, slice) entries; shared memory holds each
// warp's staged slice pair and its Slater scratch, or, for large matrices
// (27 x 27 free-particle matrices: 35 KB a warp), the scratch's hot part (LU
// and inverse) with the cold part (element and gradient matrices) in global
// memory, so that more warps stay resident.
__global__ void __launch_bounds__(kBlock) cache_prefill_kernel(PrefillParams P) {
  extern __shared__ double sh[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
  const long long gw = (long long)blockIdx.x * nwarps + warp;
  const long long nwt = (long long)gridDim.x * nwarps;
  double* st = sh + (size_t)warp * P.stage_stride;
  double* scr = P.gscratch ? P.gscratch + gw * P.scratch_stride
                           : sh + (size_t)nwarps * P.stage_stride + (size_t)warp * P.scratch_stride;
  double* cold = P.gcold ? P.gcold + gw * P.cold_stride : nullptr;
  const long long ntask = (long long)P.nslot * P.ntask_per_slot;
  for (long long task = gw; task < ntask; task += nwt) {  // warp-uniform
    const int k = (int)(task / P.ntask_per_slot), tk = (int)(task % P.ntask_per_slot);
    const int r = P.slots ? P.slots[k] : k;
    const DevSys& s = P.sys[r];
    if (s.nc_offset < 0) continue;
    const int M = s.nslice, sp = tk / M, t = tk % M;
    if (sp >= s.nspecies || !s.node_kind[sp]) continue;
    const int n = s.spec_count[sp], f = s.spec_first[sp], np = s.npart;
    const double* path = P.paths + s.path_offset;
    double* e = P.cache + s.nc_offset + ((size_t)sp * M + t) * s.nc_stride;
    const double scale = P.state[r].node_scale[sp];
    const double ep = (double)P.state[r].epoch[sp];
    if (P.only_invalid && e[0] == ep) continue;  // warp-uniform
    // stage the species' beads of slices t (r1) and t + M/2 (r2)
    const int t2 = (t + M / 2) % M;
    __syncwarp();
    for (int p = lane; p < n; p += 32) {
      const double* b1 = path + ((size_t)t * np + f + p) * 3;
      const double* b2 = path + ((size_t)t2 * np + f + p) * 3;
      st[p] = b1[0];
      st[n + p] = b1[1];
      st[2 * n + p] = b1[2];
      st[3 * n + p] = b2[0];
      st[4 * n + p] = b2[1];
      st[5 * n + p] = b2[2];
    }
    __syncwarp();
    // node_eval_group reads particle f + p: views offset so that it lands on entry p
    SliceView v1{st - f, st + n - f, st + 2 * n - f, n, 0, -1, 0, 0, 0};
    SliceView v2{st + 3 * n - f, st + 4 * n - f, st + 5 * n - f, n, 0, -1, 0, 0, 0};
    double det = 0;
    int err = 0;
    // (mixed form, free-particle nodes: the inverse block too, the start of
    // its update count)
    if (sm_species(s, sp))
      node_eval_group<32, true>(s, sp, v1, v2, scale, scr, 1, e + 2 + 2 * n, -1, true, det, err,
                                e + 2, e + 2 + n, nullptr, 0xffffffffu, cold, nullptr, 0.0,
                                e + cache_x_slot(s, sp), ep);
    else
      node_eval_group<32>(s, sp, v1, v2, scale, scr, 1, e + 2 + 2 * n, -1, true, det, err, e + 2,
                          e + 2 + n, nullptr, 0xffffffffu, cold);
    __syncwarp();
    if (lane == 0) {
      e[1] = det;
      e[0] = err ? __longlong_as_double(0x7ff8000000000000LL) : ep;
      e[cache_mask_slot(s, sp)] = 0.0;
    }
  }
}

}  // namespace pimc

namespace pimc {

// Structure factors rho_k = sum_j q_j e^{ik.r_j} of every slice of the given
// replicas (EwaldSum::evalLongRange's sum over particles,
// src/util/EwaldSum.cc:152-170), each term on the cache's fixed-point grid, so
// the integer sum is exact and independent of the order of the terms: the
// section kernel's incremental updates keep these bits.  One CTA per
// (replica, slice); the bead tables of the slice in shared memory.
struct EkPrefillParams {
  const DevSys* sys;
  const double* paths;
  long long* ek;       // the structure-factor cache pool (entries at sys.ek_offset)
  const int* slots;    // replicas to fill (null: 0 .. nslot-1)
  int nslot;
  int nslice_max;
  const unsigned char* changed;  // [replica][nslice_max]: only these slices (null: all)
};

__global__ void __launch_bounds__(kBlock) ewald_prefill_kernel(EkPrefillParams P) {
  extern __shared__ double sh[];
  const int k0 = blockIdx.y;
  const int r = P.slots ? P.slots[k0] : k0;
  const DevSys& s = P.sys[r];
  const int t = blockIdx.x;
  if (s.ek_offset < 0 || t >= s.nslice) return;
  if (P.changed && !P.changed[(size_t)r * P.nslice_max + t]) return;
  const int np = s.npart, totk = s.totk;
  const int ky0 = s.ikmax[1], kz0 = s.ikmax[2];
  const int nx = s.ikmax[0] + 1, ny = 2 * ky0 + 1;
  const int w = np;
  double2* X = (double2*)sh;
  double2* Y = X + nx * w;
  double2* Z = Y + ny * w;
  double* q = (double*)(Z + (2 * kz0 + 1) * w);
  const double* path = P.paths + s.path_offset + (size_t)t * np * 3;
  for (int j = threadIdx.x; j < np; j += blockDim.x) {
    ewald_bead_tables(s, X, Y, Z, w, j, path[3 * j], path[3 * j + 1], path[3 * j + 2]);
    q[j] = s.charge[species_of(s, j)];
  }
  __syncthreads();
  long long* out = P.ek + s.ek_offset + (size_t)t * totk * 2;
  for (int k = threadIdx.x; k < totk; k += blockDim.x) {
    const int kx = __ldg(s.kvec + 3 * k), ky = __ldg(s.kvec + 3 * k + 1) + ky0,
              kz = __ldg(s.kvec + 3 * k + 2) + kz0;
    long long re = 0, im = 0;
    for (int j = 0; j < np; ++j) {
      long long a, b;
      ewald_term_fixed(s, X, Y, Z, w, j, kx, ky, kz, q[j], a, b);
      re += a;
      im += b;
    }
    *(longlong2*)(out + 2 * k) = make_longlong2(re, im);
  }
}

}  // namespace pimc
