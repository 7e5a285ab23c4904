// The section-move sampler: shared-memory layout, section staging, mover,
// fixed-node set-up and levels, and the persistent kernel itself.
#pragma once
#include "../../include/pimc_gb300.h"
#include "section_kernel.cuh"

namespace pimc {

// Offsets (in doubles) of the shared-memory working set; computed on the host
// for the largest replica of a launch.
struct Layout {
  int s1, s2, mv, red, q, dm, ndm, dist, ndist, ewt, nodescr, ictl, ecache, ncol;
  int ncol_stride;
  int nrm;  // the attempt's normals, 3 per movable slice
  int vred;             // vector reductions: [8][kWarps] partials, then 8 sums
  int nodescr_in_smem;  // the node scratch (its hot parts when split) in shared memory
  int nodescr_stride;   // doubles per warp of that scratch
  int split;            // cold parts apart, in the CTA's global area
  int nodecold_stride;  // doubles per warp of the cold parts
  int ncol_global;      // the new-column buffer in the CTA's global area
  int gcta;             // doubles of global scratch per CTA
  int ewt_cols;         // bead columns of the Ewald tables area
  int total;  // doubles
};

struct RunParams {
  const DevSys* sys;
  DevState* state;
  double* paths;
  double* nodecache;  // per-replica Slater-result cache pool (null: none)
  double* nodescr_g;  // global per-warp node scratch when it does not fit in smem
  pimc_move_record* rec;
  const int* order;  // replicas in decreasing cost (longest first)
  int* next;         // work-queue head, zeroed before each launch
  int nattempt;
  const int* nattempt_r;  // per-replica attempts (null: nattempt for every replica)
  long long* ekcache;     // structure-factor cache pool (null: none)
  long long* ekstage;     // per-CTA staging of an attempt's new structure factors
  int ekstage_stride;     // int64 words per CTA
  double* xstage;         // mixed form: per-CTA staging of changed slices' inverses (null: none)
  long long xstage_cta;   // doubles per CTA
  int nrep;
  uint64_t seed;
  Layout lay;
};

__device__ __forceinline__ Smem carve(double* base, const Layout& L, const DevSys& s,
                                      double* nodescr_g, double* xstage = nullptr) {
  Smem m;
  // mixed form: this CTA's staging of the inverse blocks of an attempt's changed
  // slices ([nsec][2 + ns_max^2], global memory), committed to the cache on accept
  m.xstage = xstage;
  m.xstage_stride = s.ns_max * s.ns_max + 2;
  const int ss = s.nsec * s.npart;
  m.s1x = base + L.s1;
  m.s1y = m.s1x + ss;
  m.s1z = m.s1y + ss;
  m.s2x = base + L.s2;
  m.s2y = m.s2x + ss;
  m.s2z = m.s2y + ss;
  m.mx = base + L.mv;
  m.my = m.mx + s.nsec;
  m.mz = m.my + s.nsec;
  m.red = base + L.red;
  m.vred = base + L.vred;
  m.qpart = base + L.q;
  m.dm = base + L.dm;
  m.ndm = base + L.ndm;
  m.dist = base + L.dist;
  m.ndist = base + L.ndist;
  m.ewt = base + L.ewt;
  m.ictl = (int*)(base + L.ictl);
  m.ecache = L.ecache >= 0 ? base + L.ecache : nullptr;
  // the CTA's global area: per-warp node scratch (all of it, or the cold parts),
  // then the new-column buffer when it is not in shared memory
  double* gbase = nodescr_g ? nodescr_g + (size_t)blockIdx.x * L.gcta : nullptr;
  const int nw = blockDim.x >> 5;
  const int gwarp = L.split ? L.nodecold_stride : (L.nodescr_in_smem ? 0 : L.nodescr_stride);
  m.ncol = L.ncol >= 0 ? base + L.ncol
                       : ((L.ncol_global && gbase) ? gbase + (size_t)nw * gwarp : nullptr);
  m.nodecold = (L.split && gbase) ? gbase : nullptr;
  m.nodecold_stride = L.nodecold_stride;
  m.ewt_cols = L.ewt_cols;
  m.nrm = base + L.nrm;
  m.ncol_stride = L.ncol_stride;
  m.nodescr_stride = L.nodescr_stride;
  m.nodescr = L.nodescr_in_smem ? base + L.nodescr : gbase;
  return m;
}

__device__ __forceinline__ int species_of(const DevSys& s, int p) {
  int r = 0;
  for (int k = 0; k < s.nspecies; ++k)
    if (p >= s.spec_first[k] && p < s.spec_first[k] + s.spec_count[k]) r = k;
  return r;
}

// Section slice k of a section starting at ifirst, in path slice numbering with
// the identity permutation (SerialPaths::getBeads, src/base/SerialPaths.cc:119-136).
__device__ __forceinline__ int wrap_slice(int islice, int M) {
  return islice < 0 ? islice + M : (islice < M ? islice : islice - M);
}

// The level-0 Ewald term of CoulombAction::getActionDifference
// (src/action/CoulombAction.cc:107-119: evalLongRange of the new minus the old
// configuration on section slices 1 .. 2^L-1, times tau/epsilon) from the
// slices' cached structure factors: only the moving particle's term changes,
// rho'_k = rho_k + q (e^{ik.r'} - e^{ik.r}), exact on the fixed-point grid, and
// evalLongRange's difference is sum_k 2 v_k (|rho'_k|^2 - |rho_k|^2) / (2V)
// (the self energy cancels).  O(totk) per slice instead of O(totk N) for each
// of the two configurations.  rho'_k goes to `stage` for the accept step.
static __device__ __noinline__ double ewald_level0_cached(const DevSys& s, const Smem& m, int ipart,
                                             int ifirst1, const long long* ek, long long* stage) {
  const int np = s.npart, nsec = s.nsec, M = s.nslice, totk = s.totk;
  const int ky0 = s.ikmax[1], kz0 = s.ikmax[2];
  const int nx = s.ikmax[0] + 1, ny = 2 * ky0 + 1;
  const int w = m.ewt_cols;  // bead columns of the tables area
  const int chunk = w / 2;   // slices per pass: the old and the new bead of each
  double2* X = (double2*)m.ewt;
  double2* Y = X + nx * w;
  double2* Z = Y + ny * w;
  const double q = m.qpart[ipart], is = 1.0 / s.ek_scale;
  double acc = 0.0;
  for (int t0 = 1; t0 < nsec - 1; t0 += chunk) {
    const int nt = min(chunk, nsec - 1 - t0);
    __syncthreads();
    for (int c = threadIdx.x; c < 2 * nt; c += blockDim.x) {
      const int t = t0 + (c >> 1);
      if (c & 1)
        ewald_bead_tables(s, X, Y, Z, w, c, m.mx[t], m.my[t], m.mz[t]);
      else
        ewald_bead_tables(s, X, Y, Z, w, c, m.s1x[t * np + ipart], m.s1y[t * np + ipart],
                          m.s1z[t * np + ipart]);
    }
    __syncthreads();
    for (int it = threadIdx.x; it < nt * totk; it += blockDim.x) {
      const int tt = it / totk, k = it - tt * totk, t = t0 + tt;
      const int kx = __ldg(s.kvec + 3 * k), ky = __ldg(s.kvec + 3 * k + 1) + ky0,
                kz = __ldg(s.kvec + 3 * k + 2) + kz0;
      const longlong2 o =
          *(const longlong2*)(ek + ((size_t)wrap_slice(ifirst1 + t, M) * totk + k) * 2);
      long long are, aim, bre, bim;
      ewald_term_fixed(s, X, Y, Z, w, 2 * tt, kx, ky, kz, q, are, aim);
      ewald_term_fixed(s, X, Y, Z, w, 2 * tt + 1, kx, ky, kz, q, bre, bim);
      const long long nre = o.x + (bre - are), nim = o.y + (bim - aim);
      *(longlong2*)(stage + ((size_t)(t - 1) * totk + k) * 2) = make_longlong2(nre, nim);
      const double ore = __ll2double_rn(o.x) * is, oim = __ll2double_rn(o.y) * is;
      const double rre = __ll2double_rn(nre) * is, rim = __ll2double_rn(nim) * is;
      acc += 2 * __ldg(s.vk + k) * ((rre * rre + rim * rim) - (ore * ore + oim * oim));
    }
  }
  const double sum = block_sum(acc, m.red);
  return sum * s.one_over_2v * s.tau / s.epsilon;
}

static __device__ __noinline__ void load_section(const DevSys& s, const double* path, int ifirst, double* sx,
                             double* sy, double* sz) {
  const int np = s.npart, n = s.nsec * np;
  for (int idx = threadIdx.x; idx < n; idx += blockDim.x) {
    const int k = idx / np, p = idx - k * np;
    const int t = wrap_slice(ifirst + k, s.nslice);
    const double* src = path + ((size_t)t * np + p) * 3;
    sx[idx] = src[0];
    sy[idx] = src[1];
    sz[idx] = src[2];
  }
}

// SerialPaths::putBeads (src/base/SerialPaths.cc:143-185) with the identity permutation.
static __device__ __noinline__ void store_section(const DevSys& s, double* path, int ifirst, const double* sx,
                              const double* sy, const double* sz) {
  const int np = s.npart, n = s.nsec * np;
  for (int idx = threadIdx.x; idx < n; idx += blockDim.x) {
    const int k = idx / np, p = idx - k * np;
    const int islice = ifirst + k;
    if (islice < 0) continue;
    const int t = islice < s.nslice ? islice : islice % s.nslice;
    double* dst = path + ((size_t)t * np + p) * 3;
    dst[0] = sx[idx];
    dst[1] = sy[idx];
    dst[2] = sz[idx];
  }
}

// FreeMover::makeMove (src/advancer/mover/FreeMover.cc:59-124) and
// FreeMoverPBC::makeMove (src/advancer/mover/FreeMoverPBC.cc:59-152) for one
// moving particle at one level; threads own moved slices.  Returns ln(T_old/T_new).
// Every normal the attempt's mover can use, drawn in parallel before the
// levels: moved slice `ord` (0 .. 2^L - 2 in FreeMover's order) takes Box-Muller
// pairs 2 ord and 2 ord + 1 and uses the first three values.  Both precision
// forms draw the same FP64 normals, so a mixed-form chain makes the FP64
// chain's proposals and its action differences can be compared with the FP64
// form's on identical moves.
static __device__ __noinline__ void attempt_normals(const DevSys& s, const Smem& m, uint64_t seed,
                                       uint32_t rep, uint32_t att) {
  // (with delayed rejection one more: the second proposal at level nlevel - 1
  // takes order 1, the slices after it one order later)
  const int nord = (1 << s.nlevel) - 1 + (s.dr ? 1 : 0);
  for (int o = threadIdx.x; o < nord; o += blockDim.x) {
    double z0, z1, z2, z3;
    stream_normal_pair(seed, rep, att, 2u * o, &z0, &z1);
    stream_normal_pair(seed, rep, att, 2u * o + 1u, &z2, &z3);
    m.nrm[3 * o] = z0;
    m.nrm[3 * o + 1] = z1;
    m.nrm[3 * o + 2] = z2;
  }
}

// oshift: moved-slice orders taken by a delayed-rejection proposal before
// this level; second: the delayed-rejection proposal itself (its width).
static __device__ __noinline__ double mover_level_part(const DevSys& s, const Smem& m, int ipart, int level,
                              uint64_t seed, uint32_t rep, uint32_t att, uint32_t ubase,
                              int oshift = 0, bool second = false) {
  const int L = s.nlevel, np = s.npart;
  const int nStride = 1 << level;
  const int nmov = (level == L) ? 0 : (1 << (L - level - 1));
  const int ord0 = ((level == L) ? 0 : (1 << (L - level - 1)) - 1) + oshift;
  const int sp = species_of(s, ipart);
  const double sigma = second ? s.dr_sigma[sp] : s.mov_sigma[level][sp];
  const double inv2Sigma2 = second ? s.dr_inv2s2[sp] : s.mov_inv2s2[level][sp];
  double part = 0.0;
  for (int k = threadIdx.x; k < nmov; k += blockDim.x) {
    const int t = nStride * (2 * k + 1), tp = t - nStride, tn = t + nStride;
    // the attempt's normals were drawn up front (attempt_normals)
    const double z0 = m.nrm[3 * (ord0 + k)], z1 = m.nrm[3 * (ord0 + k) + 1];
    const double z2 = m.nrm[3 * (ord0 + k) + 2];
    const double ox = m.s1x[t * np + ipart], oy = m.s1y[t * np + ipart], oz = m.s1z[t * np + ipart];
    const double opx = m.s1x[tp * np + ipart], opy = m.s1y[tp * np + ipart], opz = m.s1z[tp * np + ipart];
    const double onx = m.s1x[tn * np + ipart], ony = m.s1y[tn * np + ipart], onz = m.s1z[tn * np + ipart];
    const double mpx = m.mx[tp], mpy = m.my[tp], mpz = m.mz[tp];
    const double mnx = m.mx[tn], mny = m.my[tn], mnz = m.mz[tn];
    double acc = 0.0;
    if (s.mover == PIMC_MOVER_FREE) {
      double mdx = mnx - mpx, mdy = mny - mpy, mdz = mnz - mpz;
      pbc(s, mdx, mdy, mdz);
      mdx *= 0.5; mdy *= 0.5; mdz *= 0.5;
      mdx += mpx; mdy += mpy; mdz += mpz;
      pbc(s, mdx, mdy, mdz);
      double dx = z0 * sigma, dy = z1 * sigma, dz = z2 * sigma;
      pbc(s, dx, dy, dz);
      double nx = mdx + dx, ny = mdy + dy, nz = mdz + dz;
      pbc(s, nx, ny, nz);
      m.mx[t] = nx;
      m.my[t] = ny;
      m.mz[t] = nz;
      acc += dx * dx * inv2Sigma2;
      acc += dy * dy * inv2Sigma2;
      acc += dz * dz * inv2Sigma2;
      double ax = onx - opx, ay = ony - opy, az = onz - opz;
      pbc(s, ax, ay, az);
      ax *= 0.5; ay *= 0.5; az *= 0.5;
      ax += opx; ay += opy; az += opz;
      pbc(s, ax, ay, az);
      double ex = ox - ax, ey = oy - ay, ez = oz - az;
      pbc(s, ex, ey, ez);
      acc -= ex * ex * inv2Sigma2;
      acc -= ey * ey * inv2Sigma2;
      acc -= ez * ez * inv2Sigma2;
    } else {
      double md[3] = {mnx - mpx, mny - mpy, mnz - mpz};
      pbc(s, md[0], md[1], md[2]);
      md[0] *= 0.5; md[1] *= 0.5; md[2] *= 0.5;
      double m2[3] = {md[0] + 0.5 * s.cell[0], md[1] + 0.5 * s.cell[1], md[2] + 0.5 * s.cell[2]};
      pbc(s, m2[0], m2[1], m2[2]);
      for (int d = 0; d < 3; ++d) {
        // No periodic Gaussian on the mover path (the engine rejects boxes that need one).
        const double w1 = exp(-inv2Sigma2 * md[d] * md[d]);
        const double w2 = exp(-inv2Sigma2 * m2[d] * m2[d]);
        const double u = stream_uniform(seed, rep, att, ubase + 3u * k + d);
        if (u > w1 / (w1 + w2)) md[d] = m2[d];
      }
      double nx = md[0] + mpx + z0 * sigma, ny = md[1] + mpy + z1 * sigma, nz = md[2] + mpz + z2 * sigma;
      pbc(s, nx, ny, nz);
      m.mx[t] = nx;
      m.my[t] = ny;
      m.mz[t] = nz;
      double pn[3] = {nx - mpx, ny - mpy, nz - mpz}, nn[3] = {nx - mnx, ny - mny, nz - mnz};
      double dn[3] = {mnx - mpx, mny - mpy, mnz - mpz};
      double po[3] = {ox - opx, oy - opy, oz - opz}, no[3] = {ox - onx, oy - ony, oz - onz};
      double dol[3] = {onx - opx, ony - opy, onz - opz};
      pbc(s, pn[0], pn[1], pn[2]);
      pbc(s, nn[0], nn[1], nn[2]);
      pbc(s, dn[0], dn[1], dn[2]);
      pbc(s, po[0], po[1], po[2]);
      pbc(s, no[0], no[1], no[2]);
      pbc(s, dol[0], dol[1], dol[2]);
      for (int d = 0; d < 3; ++d) {
        acc -= po[d] * po[d] * inv2Sigma2 * 0.5;
        acc -= no[d] * no[d] * inv2Sigma2 * 0.5;
        acc += pn[d] * pn[d] * inv2Sigma2 * 0.5;
        acc += nn[d] * nn[d] * inv2Sigma2 * 0.5;
        acc += dol[d] * dol[d] * inv2Sigma2 * 0.25;
        acc -= dn[d] * dn[d] * inv2Sigma2 * 0.25;
      }
    }
    part += acc;
  }
  return part;
}

// FreeMover(PBC)::makeMove for one level: the beads, and ln(T_old/T_new) summed over the block.
static __device__ double mover_level(const DevSys& s, const Smem& m, int ipart, int level,
                              uint64_t seed, uint32_t rep, uint32_t att, uint32_t ubase,
                              int oshift = 0, bool second = false) {
  return block_sum(mover_level_part(s, m, ipart, level, seed, rep, att, ubase, oshift, second),
                   m.red);
}


// Block sums of nv per-thread values (nv <= 8) in a fixed order: warp trees,
// then the warps in turn; out[v] is visible to every thread on return.
__device__ __forceinline__ void block_sum_vec(const double* v, int nv, double* buf, double* out) {
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
  for (int k = 0; k < nv; ++k) {
    double x = v[k];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (l == 0) buf[k * kWarps + w] = x;
  }
  __syncthreads();
  if (threadIdx.x < nv) {
    double x = 0.0;
    for (int i = 0; i < nw; ++i) x += buf[threadIdx.x * kWarps + i];
    out[threadIdx.x] = x;
  }
  __syncthreads();
}

// Evaluates one slice pair per lane group (group width W from the species size).
__device__ __forceinline__ void node_eval_dispatch(int W, const DevSys& s, int sp,
                                                   const SliceView& v1, const SliceView& v2,
                                                   double scale, double* scr, int full,
                                                   double* ecache, int jcol, bool write,
                                                   double& det, int& err, double* d1,
                                                   double* d2, double* newcol = nullptr,
                                                   unsigned rowmask = 0xffffffffu,
                                                   double* cold = nullptr,
                                                   const double* xin = nullptr,
                                                   double det_in = 0.0, double* xout = nullptr,
                                                   double xepoch = 0.0) {
  // (xin and xout are the same for every lane of a warp)
  if (xin || xout) {
    if (W == 8)
      node_eval_group<8, true>(s, sp, v1, v2, scale, scr, full, ecache, jcol, write, det, err,
                               d1, d2, newcol, rowmask, cold, xin, det_in, xout, xepoch);
    else if (W == 16)
      node_eval_group<16, true>(s, sp, v1, v2, scale, scr, full, ecache, jcol, write, det, err,
                                d1, d2, newcol, rowmask, cold, xin, det_in, xout, xepoch);
    else
      node_eval_group<32, true>(s, sp, v1, v2, scale, scr, full, ecache, jcol, write, det, err,
                                d1, d2, newcol, rowmask, cold, xin, det_in, xout, xepoch);
  } else if (W == 8) {
    node_eval_group<8>(s, sp, v1, v2, scale, scr, full, ecache, jcol, write, det, err, d1, d2,
                       newcol, rowmask, cold);
  } else if (W == 16) {
    node_eval_group<16>(s, sp, v1, v2, scale, scr, full, ecache, jcol, write, det, err, d1, d2,
                        newcol, rowmask, cold);
  } else {
    node_eval_group<32>(s, sp, v1, v2, scale, scr, full, ecache, jcol, write, det, err, d1, d2,
                        newcol, rowmask, cold);
  }
}

// Index of the entry's stale-row word (after the element matrices): bit r set
// = row r (r2 particle r) moved since the matrix was cached; bit 63 = the
// cached matrix is not usable at all.
__device__ __forceinline__ int cache_mask_slot(const DevSys& s, int sp) {
  const int n = s.spec_count[sp];
  return 2 + 2 * n + n * n * (s.node_kind[sp] == PIMC_NODES_FREE ? 4 : 1);
}
// Whether a species' cached Slater entries carry the inverse block that the
// mixed form's Sherman-Morrison updates work on: FreeParticleNodes species.
// (The SHONodes matrices of the cold dots are ill-conditioned by
// construction, cond 1e12..1e14 at omega/T = 20, where every factorisation
// fails the updates' conditioning gate: the block would only cost them.)
__host__ __device__ __forceinline__ bool sm_species(const DevSys& s, int sp) {
  return s.mixed && s.node_kind[sp] == PIMC_NODES_FREE;
}
// Mixed form: index of the entry's inverse block [epoch of its scale, updates
// since the last factorisation, inverse (n*n, X layout)], after the stale-row word.
__device__ __forceinline__ int cache_x_slot(const DevSys& s, int sp) {
  return cache_mask_slot(s, sp) + 1;
}
__device__ __forceinline__ unsigned cache_rowmask(const double* e, int slot) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(e[slot]);
  return (b >> 63) ? 0xffffffffu : (unsigned)(b & 0xffffffffull);
}

// Slater-result cache entry of species sp for path slice t1 (r1 at t1, r2 at
// t1 + M/2): [0] epoch (NaN = invalid), [1] determinant, [2..2+n) d1,
// [2+n..2+2n) d2, [2+2n..) exp matrix (SHONodes).  An entry is valid while
// neither slice's particles of that species have moved and the species'
// scale epoch is unchanged; evaluate() of the same inputs at the same scale
// returns exactly these values, so a hit replaces the evaluation bit for bit.
__device__ __forceinline__ double* cache_entry(const DevSys& s, double* cache, int sp, int t1) {
  return cache + ((size_t)sp * s.nslice + t1) * s.nc_stride;
}

// One pass of the set-up over slices [start, nsec) of one node species (only_sp)
// or of all of them (only_sp < 0): cached results are copied, the others are
// evaluated, the species' warps side by side.  Determinants go to dm[sp][t],
// error flags to errs[sp][t], the moving species' distances to dist.
static __device__ __noinline__ void node_init_pass(const DevSys& s, const Smem& m, const double* scale,
                                      const int* epoch, int msp, double* cache, int ifirst1,
                                      int only_sp, int start) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
  const int nsec = s.nsec, M = s.nslice, nsm = s.ns_max;
  int* errs = m.ictl + C_NCTL;                 // [kMaxSpecies][nsec]
  int* miss = errs + kMaxSpecies * nsec;       // [kMaxSpecies][nsec] slices to evaluate
  int* nmiss = m.ictl + C_NMISS;               // [kMaxSpecies] (C_NMISS .. C_NMISS + 3)
  const double NaN = __longlong_as_double(0x7ff8000000000000LL);
  if (threadIdx.x < kMaxSpecies) nmiss[threadIdx.x] = 0;
  __syncthreads();
  const int nt = nsec - start;
  for (int it = threadIdx.x; it < s.nspecies * nt; it += blockDim.x) {
    const int sp = it / nt, t = start + (it - sp * nt);
    if (!s.node_kind[sp] || (only_sp >= 0 && sp != only_sp)) continue;
    const int n = s.spec_count[sp];
    const double* e = cache ? cache_entry(s, cache, sp, wrap_slice(ifirst1 + t, M)) : nullptr;
    if (e && e[0] == (double)epoch[sp]) {
      m.dm[sp * nsec + t] = e[1];
      errs[sp * nsec + t] = 0;
      if (sp == msp)
        for (int j = 0; j < n; ++j) {
          m.dist[(t * 2) * nsm + j] = e[2 + j];
          m.dist[(t * 2 + 1) * nsm + j] = e[2 + n + j];
        }
    } else {
      miss[sp * nsec + atomicAdd(&nmiss[sp], 1)] = t;
    }
  }
  __syncthreads();
  // warp tasks: each warp takes up to G misses of one species (lane groups of
  // a warp must run the same species so that they stay converged)
  int ntask = 0;
  int Gs[kMaxSpecies], Ws[kMaxSpecies], first[kMaxSpecies + 1];
  for (int sp = 0; sp < s.nspecies; ++sp) {
    Ws[sp] = node_group_width(s.spec_count[sp]);
    Gs[sp] = 32 / Ws[sp];
    first[sp] = ntask;
    ntask += (nmiss[sp] + Gs[sp] - 1) / Gs[sp];
  }
  first[s.nspecies] = ntask;
  for (int wt = warp; wt < ntask; wt += nwarps) {
    int sp = 0;
    while (wt >= first[sp + 1]) ++sp;
    const int n = s.spec_count[sp];
    const bool sho = s.node_kind[sp] == PIMC_NODES_SHO, mine = sp == msp;
    const int W = Ws[sp], gm = lane / W, glm = lane & (W - 1);
    const int base = (wt - first[sp]) * Gs[sp];
    const int task = base + gm;
    const bool act = task < nmiss[sp];
    const int t = miss[sp * nsec + (act ? task : base)];
    double* scrm = group_scr(m, warp, gm, n, !sho);
    double* coldm = group_cold(m, warp, gm, n, !sho);
    double* e = cache ? cache_entry(s, cache, sp, wrap_slice(ifirst1 + t, M)) : nullptr;
    SliceView v1{m.s1x, m.s1y, m.s1z, s.npart, t, -1, 0, 0, 0};
    SliceView v2{m.s2x, m.s2y, m.s2z, s.npart, t, -1, 0, 0, 0};
    double det = 0;
    int err = 0;
    double* ec = e ? e + 2 + 2 * n
                   : ((sho && mine && m.ecache) ? m.ecache + (size_t)t * n * n : nullptr);
    // with a cache every miss is evaluated in full so that its entry is complete
    const int full = (mine || e) ? 1 : 0;
    double* d1 = mine ? m.dist + (t * 2) * nsm : (e ? e + 2 : nullptr);
    double* d2 = mine ? m.dist + (t * 2 + 1) * nsm : (e ? e + 2 + n : nullptr);
    const unsigned rmask = e ? cache_rowmask(e, cache_mask_slot(s, sp)) : 0xffffffffu;
    // mixed form: the entry's inverse, updated for its changed rows when it can be
    double* xb = (e && sm_species(s, sp)) ? e + cache_x_slot(s, sp) : nullptr;
    node_eval_dispatch(W, s, sp, v1, v2, scale[sp], scrm, full, ec, -1, act, det, err, d1, d2,
                       nullptr, rmask, coldm, xb, e ? e[1] : 0.0, xb, (double)epoch[sp]);
    if (act) {
      if (e && mine && glm < n) {
        e[2 + glm] = d1[glm];
        e[2 + n + glm] = d2[glm];
      }
      if (glm == 0) {
        m.dm[sp * nsec + t] = det;
        errs[sp * nsec + t] = err;
        if (e) {
          e[1] = det;
          e[0] = err ? NaN : (double)epoch[sp];
          e[cache_mask_slot(s, sp)] = 0.0;  // the element matrix is whole again
        }
      }
    }
  }
  __syncthreads();
}

// FixedNodeAction::initialize (src/fixednode/FixedNodeAction.cc:331-357) for every
// species with a node model, reproducing NodeModel::evaluate's rescaling loop
// (src/fixednode/SHONodes.cc:112-126): every species' slices are evaluated in
// parallel at the current scales (pi-qmc sets the species up one after the
// other; they are independent); at a species' first slice whose determinant
// leaves [1e-50, 1e50] its loop is replayed sequentially, and its later
// slices are re-evaluated.
static __device__ __noinline__ void node_initialize(const DevSys& s, const Smem& m, double* scale, int* epoch,
                                int msp, uint32_t* status, double* cache, int ifirst1) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nsec = s.nsec, M = s.nslice;
  const int nsm = s.ns_max;
  int* errs = m.ictl + C_NCTL;  // [kMaxSpecies][nsec]
  const double NaN = __longlong_as_double(0x7ff8000000000000LL);
  node_init_pass(s, m, scale, epoch, msp, cache, ifirst1, -1, 0);
  for (int sp = 0; sp < s.nspecies; ++sp) {
    if (!s.node_kind[sp]) continue;
    const int n = s.spec_count[sp];
    const int W = node_group_width(n), g = lane / W;
    const bool sho = s.node_kind[sp] == PIMC_NODES_SHO;
    const bool mine = sp == msp;
    double* dm = m.dm + sp * nsec;
    int* er = errs + sp * nsec;
    int start = 0;
    for (int round = 0; round < 64; ++round) {
      if (round > 0) node_init_pass(s, m, scale, epoch, msp, cache, ifirst1, sp, start);
      if (threadIdx.x == 0) {
        int k = -1;
        for (int t = start; t < nsec; ++t) {
          const double a = fabs(dm[t]);
          if (er[t] || a < 1e-50 || a > 1e50) {
            k = t;
            break;
          }
        }
        m.ictl[C_SCANK] = k;
      }
      __syncthreads();
      const int k = m.ictl[C_SCANK];
      if (k < 0) break;
      if (warp == 0) {
        // pi-qmc's do-while rescale loop on slice k, by group 0 of warp 0
        // (the other groups repeat it without storing).
        double det = dm[k];
        int err = er[k];
        double sc2 = scale[sp];
        int guard = 0;
        double* dsc = group_scr(m, warp, g, n, !sho);
        double* dcold = group_cold(m, warp, g, n, !sho);
        while (err || fabs(det) < 1e-50 || fabs(det) > 1e50) {
          if (err || ++guard > 2000) {
            if (lane == 0) *status |= err ? (PIMC_STATUS_SINGULAR | PIMC_STATUS_RESCALE_LIMIT)
                                          : PIMC_STATUS_RESCALE_LIMIT;
            break;
          }
          if (fabs(det) < 1e-250)
            sc2 *= 2;
          else
            sc2 *= pow(fabs(det), -1. / n);
          SliceView v1{m.s1x, m.s1y, m.s1z, s.npart, k, -1, 0, 0, 0};
          SliceView v2{m.s2x, m.s2y, m.s2z, s.npart, k, -1, 0, 0, 0};
          double d = 0;
          int e2 = 0;
          node_eval_dispatch(W, s, sp, v1, v2, sc2, dsc, mine ? 1 : 0, nullptr, -1, g == 0, d,
                             e2, m.dist + (k * 2) * nsm, m.dist + (k * 2 + 1) * nsm, nullptr,
                             0xffffffffu, dcold);
          det = __shfl_sync(0xffffffffu, d, 0);
          err = __shfl_sync(0xffffffffu, e2, 0);
        }
        if (lane == 0) {
          dm[k] = det;
          er[k] = err;
          if (sc2 != scale[sp]) epoch[sp] += 1;
          scale[sp] = sc2;
          if (cache) cache_entry(s, cache, sp, wrap_slice(ifirst1 + k, M))[0] = NaN;
        }
      }
      __syncthreads();
      start = k + 1;
      if (start >= nsec) break;
    }
    // crossing check, as the reference counts errors at set-up
    if (threadIdx.x == 0) {
      for (int t = 0; t < nsec; ++t)
        if (er[t] || dm[t] * dm[0] <= 1e-200) *status |= PIMC_STATUS_INIT_CROSSING;
    }
  }
  if (msp >= 0 && s.node_kind[msp]) {
    // newDist(0) = dist(0)
    for (int i = threadIdx.x; i < 2 * nsm; i += blockDim.x) m.ndist[i] = m.dist[i];
  }
  __syncthreads();
}

// FixedNodeAction::getActionDifference (src/fixednode/FixedNodeAction.cc:39-131)
// for the moving species at one level.
static __device__ __noinline__ double node_level(const DevSys& s, const Smem& m, double scale, int msp, int ipart,
                             int level, double* cache, int ifirst1, int ep) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
  const int nsec = s.nsec, nsm = s.ns_max;
  const int nStride = 1 << (level + 1);
  const int n = s.spec_count[msp];
  const int ntask = (nsec - 1 - nStride / 2) / nStride + 1;
  if (nStride / 2 == nsec - 1) {
    // The top level's only slice is the section's fixed end: its Slater
    // matrix is the set-up one, so its determinant and distances are copied.
    const int t = nsec - 1;
    for (int i = threadIdx.x; i < 2 * nsm; i += blockDim.x) m.ndist[t * 2 * nsm + i] = m.dist[t * 2 * nsm + i];
    if (threadIdx.x == 0) {
      m.ndm[t] = m.dm[msp * nsec + t];
      m.ictl[C_FLAG] = (m.ndm[t] * m.dm[msp * nsec + 0] <= 1e-200) ? 1 : 0;
    }
    __syncthreads();
    return m.ictl[C_FLAG] ? 2e100 : 0.0;
  }
  // lane groups of the species' width, packed (32 / W matrices a warp): the
  // SM's narrow FP64 pipe, shared by every resident warp, is the limit, and a
  // packed warp instruction serves several matrices
  const int W = node_group_width(n), G = 32 / W, g = lane / W;
  const bool sho = s.node_kind[msp] == PIMC_NODES_SHO;
  double* scr = group_scr(m, warp, g, n, !sho);
  double* cold = group_cold(m, warp, g, n, !sho);
  const int jcol = ipart - s.spec_first[msp];
  if (threadIdx.x == 0) m.ictl[C_FLAG] = 0;
  __syncthreads();
  for (int base = warp * G; base < ntask; base += nwarps * G) {
    const int task = base + g;
    const bool act = task < ntask;
    const int t = nStride / 2 + (act ? task : base) * nStride;
    SliceView v1{m.s1x, m.s1y, m.s1z, s.npart, t, ipart, m.mx[t], m.my[t], m.mz[t]};
    SliceView v2{m.s2x, m.s2y, m.s2z, s.npart, t, -1, 0, 0, 0};
    double det = 0;
    int err = 0;
    double* ec = nullptr;
    const double* xb = nullptr;  // mixed form: the entry's inverse block
    double det_in = 0.0;
    if (cache) {
      double* e = cache_entry(s, cache, msp, wrap_slice(ifirst1 + t, s.nslice));
      ec = e + 2 + 2 * n;
      if (sm_species(s, msp) && m.xstage) {
        xb = e + cache_x_slot(s, msp);
        det_in = e[1];
      }
    } else if (sho && m.ecache) {
      ec = m.ecache + (size_t)t * n * n;
    }
    node_eval_dispatch(W, s, msp, v1, v2, scale, scr, 1, ec, jcol, act, det, err,
                       m.ndist + (t * 2) * nsm, m.ndist + (t * 2 + 1) * nsm,
                       cache ? m.ncol + t * m.ncol_stride : nullptr, 0u, cold, xb, det_in,
                       xb ? m.xstage + (size_t)t * m.xstage_stride : nullptr, (double)ep);
    if (act && (lane & (W - 1)) == 0) {
      m.ndm[t] = det;
      if (err || det * m.dm[msp * nsec + 0] <= 1e-200) atomicOr(&m.ictl[C_FLAG], 1);
    }
  }
  __syncthreads();
  if (m.ictl[C_FLAG]) return 2e100;
  if (level != 0) return 0.0;
  double part = 0.0;
  FSum fpart;
  for (int it = threadIdx.x; it < (nsec - 1) * n; it += blockDim.x) {
    const int t = 1 + it / n, p = it % n;
    const double* D0 = m.dist + (t * 2) * nsm;
    const double* Dp0 = m.dist + ((t - 1) * 2) * nsm;
    const double* N0 = m.ndist + (t * 2) * nsm;
    const double* Np0 = m.ndist + ((t - 1) * 2) * nsm;
    if (s.mixed) {
      // FP32 terms (1 - e^-x through expm1 keeps them accurate near the node),
      // their sum compensated
      const float a1 = -expm1f(-(float)(D0[p] * Dp0[p]));
      const float b1 = -expm1f(-(float)(N0[p] * Np0[p]));
      const float a2 = -expm1f(-(float)(D0[nsm + p] * Dp0[nsm + p]));
      const float b2 = -expm1f(-(float)(N0[nsm + p] * Np0[nsm + p]));
      fpart.add(logf(a1) - logf(b1));
      fpart.add(logf(a2) - logf(b2));
      continue;
    }
    double a = log((1 - exp(-D0[p] * Dp0[p])) / (1 - exp(-N0[p] * Np0[p])));
    a += log((1 - exp(-D0[nsm + p] * Dp0[nsm + p])) / (1 - exp(-N0[nsm + p] * Np0[nsm + p])));
    part += a;
  }
  return block_sum(s.mixed ? fpart.value() : part, m.red);
}

// The uniform-stream index of the first uniform consumed at `level`
// (image choices of FreeMoverPBC, then the Metropolis uniform).
__device__ __forceinline__ uint32_t level_uniform_base(const DevSys& s, int level) {
  uint32_t u = (s.fixed_node ? 2u : 1u) + 1u;  // section choice + particle choice
  const uint32_t pbcu = s.mover == PIMC_MOVER_FREE_PBC ? 3u : 0u;
  for (int l = s.nlevel; l > level; --l) {
    const uint32_t nmov = (l == s.nlevel) ? 0u : (1u << (s.nlevel - l - 1));
    u += pbcu * nmov + 1u;
  }
  return u;
}

// The top bisection levels lo .. hi (all above 0) at once: the movers, level
// by level (a level's midpoints are the beads of the levels above), then the
// changed slices of every level in the range on the first warps, side by side,
// while the remaining warps compute the levels' action differences (a level's
// proposal does not depend on the decisions above it).  Per level l: lds[l]
// the action difference, llt[l] the mover's ln(T_old/T_new), lnd[l] the
// fixed-node difference (2e100 when a changed slice crosses a node, else 0).
// The caller applies pi-qmc's level-by-level decisions to them.
static __device__ __noinline__ void top_levels(const DevSys& s, const Smem& m, double scale, int msp,
                                  int ipart, int lo, int hi, bool mynode, double* cache,
                                  int ifirst1, int ep, uint64_t seed, uint32_t att, double* lds,
                                  double* llt, double* lnd) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
  const int nsec = s.nsec, nsm = s.ns_max, L = s.nlevel;
  // hi - lo + 1 <= 4 levels: v[0..3] mover terms, v[4..7] action terms
  double v[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (int level = hi; level >= lo; --level) {
    const double p = mover_level_part(s, m, ipart, level, seed, s.stream_id, att,
                                      level_uniform_base(s, level));
#pragma unroll
    for (int k = 0; k < 4; ++k)
      if (k == hi - level) v[k] = p;
    __syncthreads();  // this level's beads before the next level's midpoints
  }
  const int n = mynode ? s.spec_count[msp] : 1;
  const int top = hi == L ? L - 1 : hi;
  int ntask = 0;
  if (mynode)
    for (int l = top; l >= lo; --l) ntask += (nsec - 1 - (1 << l)) / (1 << (l + 1)) + 1;
  const int W = node_group_width(n), G = 32 / W, g = lane / W;
  const int nodeW = min(nwarps, (ntask + G - 1) / G);
  if (threadIdx.x == 0) m.ictl[C_FLAG] = 0;
  if (mynode && hi == L) {
    // the top level's only slice is the section's fixed end: copied from the set-up
    const int t = nsec - 1;
    for (int i = threadIdx.x; i < 2 * nsm; i += blockDim.x) m.ndist[t * 2 * nsm + i] = m.dist[t * 2 * nsm + i];
  }
  __syncthreads();
  if (mynode && hi == L && threadIdx.x == 0) {
    const int t = nsec - 1;
    m.ndm[t] = m.dm[msp * nsec + t];
    if (m.ndm[t] * m.dm[msp * nsec + 0] <= 1e-200) atomicOr(&m.ictl[C_FLAG], 1 << L);
  }
  if (warp < nodeW) {
    const bool sho = s.node_kind[msp] == PIMC_NODES_SHO;
    double* scr = group_scr(m, warp, g, n, !sho);
    double* cold = group_cold(m, warp, g, n, !sho);
    const int jcol = ipart - s.spec_first[msp];
    for (int base = warp * G; base < ntask; base += nodeW * G) {
      const int task = base + g;
      const bool act = task < ntask;
      int k = act ? task : base, l = top;  // task -> (level, slice)
      for (;;) {
        const int nl = (nsec - 1 - (1 << l)) / (1 << (l + 1)) + 1;
        if (k < nl || l == lo) break;
        k -= nl;
        --l;
      }
      const int t = (1 << l) + k * (1 << (l + 1));
      SliceView v1{m.s1x, m.s1y, m.s1z, s.npart, t, ipart, m.mx[t], m.my[t], m.mz[t]};
      SliceView v2{m.s2x, m.s2y, m.s2z, s.npart, t, -1, 0, 0, 0};
      double det = 0;
      int err = 0;
      double* ec = nullptr;
      const double* xb = nullptr;  // mixed form: the entry's inverse block
      double det_in = 0.0;
      if (cache) {
        double* e = cache_entry(s, cache, msp, wrap_slice(ifirst1 + t, s.nslice));
        ec = e + 2 + 2 * n;
        if (sm_species(s, msp) && m.xstage) {
          xb = e + cache_x_slot(s, msp);
          det_in = e[1];
        }
      } else if (sho && m.ecache) {
        ec = m.ecache + (size_t)t * n * n;
      }
      node_eval_dispatch(W, s, msp, v1, v2, scale, scr, 1, ec, jcol, act, det, err,
                         m.ndist + (t * 2) * nsm, m.ndist + (t * 2 + 1) * nsm,
                         cache ? m.ncol + t * m.ncol_stride : nullptr, 0u, cold, xb, det_in,
                         xb ? m.xstage + (size_t)t * m.xstage_stride : nullptr, (double)ep);
      if (act && (lane & (W - 1)) == 0) {
        m.ndm[t] = det;
        if (err || det * m.dm[msp * nsec + 0] <= 1e-200) atomicOr(&m.ictl[C_FLAG], 1 << l);
      }
    }
  }
  // the action differences on the other warps (on all of them when the node
  // tasks take every warp, after those)
  if (nodeW == nwarps) __syncthreads();
  const int a0 = nodeW == nwarps ? 0 : nodeW * 32;
  if ((int)threadIdx.x >= a0)
    for (int level = lo; level <= hi; ++level) {
      const double a = action_partial(s, m, ipart, level, threadIdx.x - a0, blockDim.x - a0);
#pragma unroll
      for (int k = 0; k < 4; ++k)
        if (k == level - lo) v[4 + k] = a;
    }
  __syncthreads();
  const int flags = m.ictl[C_FLAG];
  double* out = m.vred + 8 * kWarps;
  block_sum_vec(v, 8, m.vred, out);
  if (threadIdx.x == 0)
    for (int level = lo; level <= hi; ++level) {
      llt[level] = out[hi - level];
      lds[level] = out[4 + level - lo];
      lnd[level] = ((flags >> level) & 1) ? 2e100 : 0.0;
    }
  __syncthreads();
}


// MultiLevelSampler::tryMove's delayed rejection (src/advancer/MultiLevelSampler.cc:114-148;
// DoubleMLSampler.cc:148-204 with the node term) after the first proposal B at
// level L - 1 was rejected: the second proposal C (width newSigmaFactor, the
// next normals), its action difference, FreeMover::makeDelayedMove
// (src/advancer/mover/FreeMover.cc:127-185) for the forward C->B and reverse
// B->C probabilities, and the combined acceptance with the next uniform.
// Thread 0 holds piRatioBoA and the acceptance of B in red[kWarps + 3, 4];
// returns the level-(L - 1) rejection (C_REJECT) and, when C is accepted, the
// modified action difference in red[kWarps + 2].
static __device__ __noinline__ void delayed_rejection(const DevSys& s, const Smem& m, double scale,
                                                     int msp, int ipart, bool mynode,
                                                     double* cache, int ifirst1, int ep,
                                                     uint64_t seed, uint32_t att, uint32_t uacc,
                                                     double oldDS, long long* ek,
                                                     long long* ekstage, pimc_move_record* rec,
                                                     uint32_t* status) {
  const int L = s.nlevel, level = L - 1, nsec = s.nsec;
  const int t = 1 << level, tp = 0, tn = nsec - 1;
  const int sp = species_of(s, ipart);
  double* bead = m.red + kWarps + 5;  // the rejected bead B
  if (threadIdx.x == 0) {
    bead[0] = m.mx[t];
    bead[1] = m.my[t];
    bead[2] = m.mz[t];
  }
  __syncthreads();
  // C: FreeMover::makeMove with factor = newFactor and the next normals
  const double lnTC = mover_level(s, m, ipart, level, seed, s.stream_id, att, uacc, 1, true);
  double dsC = block_sum(action_partial(s, m, ipart, level, threadIdx.x, blockDim.x), m.red);
  if (s.ewald && s.coulomb && level == 0) {
    if (ek)
      dsC += ewald_level0_cached(s, m, ipart, ifirst1, ek, ekstage);
    else
      for (int k = 1; k < nsec - 1; ++k) dsC += ewald_slice_diff(s, m, ipart, k);
  }
  double dsnC = 0.0;
  if (mynode) dsnC = node_level(s, m, scale, msp, ipart, level, cache, ifirst1, ep);
  if (threadIdx.x == 0) {
    const double piRatioBoA = m.red[kWarps + 3], accRatioA2B = m.red[kWarps + 4];
    const double sigma = s.mov_sigma[level][sp], inv2Sigma2 = s.mov_inv2s2[level][sp];
    // transA2B = B's forward probability: its Gaussian step, as makeMove drew it
    double dx = m.nrm[0] * sigma, dy = m.nrm[1] * sigma, dz = m.nrm[2] * sigma;
    pbc(s, dx, dy, dz);
    double transA2B = 0.0;
    transA2B += dx * dx * inv2Sigma2;
    transA2B += dy * dy * inv2Sigma2;
    transA2B += dz * dz * inv2Sigma2;
    transA2B += log(1.0);
    const double deltaC = s.fixed_node ? dsC + dsnC : dsC;
    const double piRatioCoA = -deltaC + oldDS;
    const double accRatioA2C = exp(lnTC + piRatioCoA);
    // makeDelayedMove with factor = defaultFactor: the midpoint of the level's
    // neighbours (the section ends, the same for B and C), B and C about it
    double mx = m.mx[tn] - m.mx[tp], my = m.my[tn] - m.my[tp], mz = m.mz[tn] - m.mz[tp];
    pbc(s, mx, my, mz);
    mx *= 0.5; my *= 0.5; mz *= 0.5;
    mx += m.mx[tp]; my += m.my[tp]; mz += m.mz[tp];
    pbc(s, mx, my, mz);
    double bx = bead[0] - mx, by = bead[1] - my, bz = bead[2] - mz;
    pbc(s, bx, by, bz);
    double forwardProb = 0.0, toldOverTnew = 0.0, tmp;
    tmp = bx * bx * inv2Sigma2; forwardProb -= tmp; toldOverTnew += tmp;
    tmp = by * by * inv2Sigma2; forwardProb -= tmp; toldOverTnew += tmp;
    tmp = bz * bz * inv2Sigma2; forwardProb -= tmp; toldOverTnew += tmp;
    forwardProb += log(1.0);
    double cx = m.mx[t] - mx, cy = m.my[t] - my, cz = m.mz[t] - mz;
    pbc(s, cx, cy, cz);
    toldOverTnew -= cx * cx * inv2Sigma2;
    toldOverTnew -= cy * cy * inv2Sigma2;
    toldOverTnew -= cz * cz * inv2Sigma2;
    toldOverTnew += log(1.0);
    const double transC2B = forwardProb;
    double accRatioC2B = exp(toldOverTnew - piRatioCoA + piRatioBoA);
    accRatioC2B = (accRatioC2B >= 1) ? 1 : accRatioC2B;
    const double accRatioA2B2C = accRatioA2C * exp(transC2B + transA2B) * (1 - accRatioC2B) /
                                 (1 - accRatioA2B);
    const double delta =
        deltaC - transC2B - transA2B - log((1 - accRatioC2B) / (1 - accRatioA2B));
    if (rec) {
      rec->ds[level] = dsC;
      rec->ds_node[level] = dsnC;
      rec->lnt[level] = lnTC;
    }
    if (!(isfinite(lnTC) && isfinite(dsC))) *status |= PIMC_STATUS_NONFINITE;
    const double u = stream_uniform(seed, s.stream_id, att, uacc + 1u);
    m.ictl[C_REJECT] = (u > accRatioA2B2C) ? level : -1;
    m.red[kWarps + 2] = delta;
  }
  __syncthreads();
}


// NT (largest block) and MINB set the register budget, 65536 / (NT * MINB)
// per thread; the variants are compiled in separate translation units
// (section_variants.cu) and chosen at run time by the launch configuration.
// kNodes = false: the variant for launches without node models, whose code
// leaves the fixed-node phases out (a smaller kernel: fewer instruction-fetch
// stalls when thousands of one-warp CTAs run different phases).
template <int NT, int MINB, bool kNodes = true>
__global__ void __launch_bounds__(NT, MINB) section_moves_kernel(RunParams P) {
  extern __shared__ double smem[];
  __shared__ DevSys S;
  __shared__ double scale[kMaxSpecies];
  __shared__ int epoch[kMaxSpecies];
  __shared__ uint32_t status;
  __shared__ long long nacc;
  __shared__ int rnext;
  // The carved pointers live in shared memory: the called phases take them
  // by reference, which would otherwise place them in each thread's stack.
  __shared__ Smem M_;
  // Persistent CTAs take replicas from a queue ordered longest-first, so that
  // uneven replicas (different N, M, L) balance across the SMs.
  for (;;) {
    if (threadIdx.x == 0) {
      const int k = atomicAdd(P.next, 1);
      rnext = (k < P.nrep) ? P.order[k] : -1;
    }
    __syncthreads();
    const int r = rnext;
    if (r < 0) break;
    {
      const int* src = (const int*)(P.sys + r);
      int* dst = (int*)&S;
      for (int i = threadIdx.x; i < (int)(sizeof(DevSys) / sizeof(int)); i += blockDim.x)
        dst[i] = src[i];
    }
    if (threadIdx.x == 0) {
      M_ = carve(smem, P.lay, P.sys[r], P.nodescr_g,
                 P.xstage ? P.xstage + (size_t)blockIdx.x * P.xstage_cta : nullptr);
      status = P.state[r].status;
      nacc = 0;
      for (int k = 0; k < kMaxSpecies; ++k) {
        scale[k] = P.state[r].node_scale[k];
        epoch[k] = P.state[r].epoch[k];
      }
    }
    __syncthreads();
    const DevSys& s = S;
    const Smem& m = M_;
    double* path = P.paths + s.path_offset;
    const uint32_t att0 = P.state[r].attempt;
    double* cache = (P.nodecache && s.nc_offset >= 0) ? P.nodecache + s.nc_offset : nullptr;
    long long* ek = (P.ekcache && s.ek_offset >= 0) ? P.ekcache + s.ek_offset : nullptr;
    long long* ekstage = ek ? P.ekstage + (size_t)blockIdx.x * P.ekstage_stride : nullptr;
    const int np = s.npart, nsec = s.nsec, M = s.nslice, L = s.nlevel;
    const bool fixed = kNodes && s.fixed_node;
    for (int i = threadIdx.x; i < np; i += blockDim.x) m.qpart[i] = s.charge[species_of(s, i)];
    const int nat = P.nattempt_r ? P.nattempt_r[r] : P.nattempt;
    for (int a = 0; a < nat; ++a) {
      const uint32_t att = att0 + (uint32_t)a;
      // ---- section choice and moving particle
      if (threadIdx.x == 0) {
        int i1, i2 = -2;
        uint32_t ui = 0;
        const double x = stream_uniform(P.seed, s.stream_id, att, ui++) * (1 - 1e-8);
        if (!fixed) {
          const int ilo = -1, ihi = M - 1;
          i1 = ilo + (int)((ihi + 1 - ilo) * x);
          if (i1 > ihi) i1 = ihi;
        } else {
          const int ilo = -1, ihi = M / 2 - 1;
          i1 = ilo + (int)((ihi + 1 - ilo) * x);
          if (i1 > ihi) i1 = ihi;
          if (stream_uniform(P.seed, s.stream_id, att, ui++) >= 0.5) i1 = (i1 + M / 2 + 1) % M - 1;
          i2 = (i1 + M / 2 + 1) % M - 1;
        }
        int ip = (int)(np * stream_uniform(P.seed, s.stream_id, att, ui++));
        if (ip >= np) ip = np - 1;
        m.ictl[C_IFIRST1] = i1;
        m.ictl[C_IFIRST2] = i2;
        m.ictl[C_IPART] = ip;
        m.ictl[C_REJECT] = -1;
      }
      __syncthreads();
      const int ifirst1 = m.ictl[C_IFIRST1], ifirst2 = m.ictl[C_IFIRST2];
      const int ipart = m.ictl[C_IPART];
      load_section(s, path, ifirst1, m.s1x, m.s1y, m.s1z);
      if (fixed) load_section(s, path, ifirst2, m.s2x, m.s2y, m.s2z);
      attempt_normals(s, m, P.seed, s.stream_id, att);
      __syncthreads();
      for (int t = threadIdx.x; t < nsec; t += blockDim.x) {
        m.mx[t] = m.s1x[t * np + ipart];
        m.my[t] = m.s1y[t * np + ipart];
        m.mz[t] = m.s1z[t * np + ipart];
      }
      const int msp = species_of(s, ipart);
      const bool mynode = fixed && s.node_kind[msp];
      if (fixed)
        node_initialize(s, m, scale, epoch, mynode ? msp : -1, &status, cache, ifirst1);
      __syncthreads();
      pimc_move_record* rec = P.rec ? P.rec + (size_t)r * P.nattempt + a : nullptr;
      double oldDS = 0.0;
      int reject = -1;
      // The top levels (L down to lb) are proposed and evaluated together,
      // their Slater matrices side by side; the decisions then follow level by
      // level exactly as below.  Work done for levels under a rejection is
      // discarded.
      // (with delayed rejection every level is taken in turn: a second proposal
      // at level L - 1 changes the normals and uniforms of the levels under it)
      const int lb = (L >= 2 && !s.dr) ? max(1, L - 3) : L + 1;
      if (lb <= L) {
        double* lds = m.red + kWarps + 8;  // [kMaxLevels] per level: action difference,
        double* llt = lds + kMaxLevels;     // mover ln T,
        double* lnd = llt + kMaxLevels;     // fixed-node difference
        top_levels(s, m, scale[msp], msp, ipart, lb, L, mynode, cache, ifirst1, epoch[msp], P.seed,
                   att, lds, llt, lnd);
        __syncthreads();
        if (threadIdx.x < 32) {
          // Lane i takes level L - i: every level's acceptance probability
          // exp(lnT - total + total of the level above) and uniform at once
          // (the same operations as one level after the other); the first
          // rejecting level from the top decides, and only the levels down to
          // it count as evaluated.
          const int lane = threadIdx.x, level = L - lane;
          const bool mine = level >= lb;
          double total = 0.0, ds = 0.0, dsn = 0.0, lnT = 0.0;
          bool rej = false;
          if (mine) {
            ds = lds[level];
            dsn = lnd[level];
            lnT = llt[level];
            total = fixed ? ds + dsn : ds;
            const double old =
                level == L ? 0.0 : (fixed ? lds[level + 1] + lnd[level + 1] : lds[level + 1]);
            const uint32_t ubase = level_uniform_base(s, level);
            const uint32_t nmov = (level == L) ? 0u : (1u << (L - level - 1));
            const uint32_t uacc = ubase + (s.mover == PIMC_MOVER_FREE_PBC ? 3u * nmov : 0u);
            const double p = exp(lnT + (-total + old));
            const double u = stream_uniform(P.seed, s.stream_id, att, uacc);
            rej = u > p;
          }
          const unsigned rmask = __ballot_sync(0xffffffffu, rej);
          const int last = rmask ? __ffs(rmask) - 1 : L - lb;  // lowest evaluated lane's index
          const bool evaluated = mine && lane <= last;
          if (evaluated && rec) {
            rec->ds[level] = ds;
            rec->ds_node[level] = dsn;
            rec->lnt[level] = lnT;
          }
          const bool bad = evaluated && !(isfinite(lnT) && isfinite(ds));
          if (__ballot_sync(0xffffffffu, bad) && lane == 0) status |= PIMC_STATUS_NONFINITE;
          if (lane == last) {
            if (rmask) m.ictl[C_REJECT] = level;
            m.red[kWarps + 2] = total;
          }
        }
        __syncthreads();
        reject = m.ictl[C_REJECT];
        oldDS = m.red[kWarps + 2];
      }
      int oshift = 0;   // moved-slice orders and uniforms a delayed-rejection
      uint32_t ushift = 0;  // proposal took before the level
      for (int level = min(L, lb - 1); level >= 0 && reject < 0; --level) {
        const uint32_t ubase = level_uniform_base(s, level) + ushift;
        const double lnT = mover_level(s, m, ipart, level, P.seed, s.stream_id, att, ubase, oshift);
        double ds = block_sum(action_partial(s, m, ipart, level, threadIdx.x, blockDim.x), m.red);
        if (s.ewald && s.coulomb && level == 0) {
          if (ek)
            ds += ewald_level0_cached(s, m, ipart, ifirst1, ek, ekstage);
          else
            for (int t = 1; t < nsec - 1; ++t) ds += ewald_slice_diff(s, m, ipart, t);
        }
        double dsn = 0.0;
        if (mynode) dsn = node_level(s, m, scale[msp], msp, ipart, level, cache, ifirst1, epoch[msp]);
        if (threadIdx.x == 0) {
          const double total = fixed ? ds + dsn : ds;
          const uint32_t nmov = (level == L) ? 0u : (1u << (L - level - 1));
          const uint32_t uacc =
              ubase + (s.mover == PIMC_MOVER_FREE_PBC ? 3u * nmov : 0u);
          const double p = exp(lnT + (-total + oldDS));
          const double u = stream_uniform(P.seed, s.stream_id, att, uacc);
          if (rec) {
            rec->ds[level] = ds;
            rec->ds_node[level] = dsn;
            rec->lnt[level] = lnT;
          }
          if (!(isfinite(lnT) && isfinite(ds))) status |= PIMC_STATUS_NONFINITE;
          if (u > p) m.ictl[C_REJECT] = level;
          m.red[kWarps + 2] = total;
          m.red[kWarps + 3] = -total + oldDS;  // piRatioBoA
          m.red[kWarps + 4] = p;               // accRatioA2B
        }
        __syncthreads();
        reject = m.ictl[C_REJECT];
        if (reject == L - 1 && s.dr) {
          const uint32_t nmov = 1u << (L - level - 1);
          const uint32_t uacc = ubase + (s.mover == PIMC_MOVER_FREE_PBC ? 3u * nmov : 0u);
          delayed_rejection(s, m, scale[msp], msp, ipart, mynode, cache, ifirst1, epoch[msp],
                            P.seed, att, uacc, oldDS, ek, ekstage, rec, &status);
          reject = m.ictl[C_REJECT];
          oshift = 1;
          ushift = 1;
        }
        if (reject >= 0) break;
        oldDS = m.red[kWarps + 2];
      }
      if (reject < 0) {
        for (int t = threadIdx.x; t < nsec; t += blockDim.x) {
          m.s1x[t * np + ipart] = m.mx[t];
          m.s1y[t * np + ipart] = m.my[t];
          m.s1z[t * np + ipart] = m.mz[t];
        }
        if (threadIdx.x == 0) ++nacc;
        if (ek) {  // the moved slices' structure factors: the staged level-0 values
          const int totk = s.totk;
          for (int it = threadIdx.x; it < (nsec - 2) * totk; it += blockDim.x) {
            const int tt = it / totk, k = it - tt * totk;
            *(longlong2*)(ek + ((size_t)wrap_slice(ifirst1 + 1 + tt, M) * totk + k) * 2) =
                *(const longlong2*)(ekstage + (size_t)it * 2);
          }
        }
        if (cache && mynode) {
          // The moved slices now hold the level evaluations; the entries that
          // pair them the other way round (r2 on a moved slice) are stale.
          const int n = s.spec_count[msp], jcol = ipart - s.spec_first[msp];
          const int nsm = s.ns_max;
          const double NaN = __longlong_as_double(0x7ff8000000000000LL);
          const bool sho = s.node_kind[msp] == PIMC_NODES_SHO;
          for (int it = threadIdx.x; it < (nsec - 2) * n; it += blockDim.x) {
            const int k = 1 + it / n, j = it % n;
            const int t1 = wrap_slice(ifirst1 + k, M);
            double* e = cache_entry(s, cache, msp, t1);
            e[2 + j] = m.ndist[(k * 2) * nsm + j];
            e[2 + n + j] = m.ndist[(k * 2 + 1) * nsm + j];
            const double* nc = m.ncol + k * m.ncol_stride;
            e[2 + 2 * n + jcol * n + j] = nc[j];
            if (!sho)
              for (int c = 1; c < 4; ++c) e[2 + 2 * n + c * n * n + jcol * n + j] = nc[c * n + j];
          }
          if (sm_species(s, msp) && m.xstage) {
            // the moved slices' inverse blocks, as the level evaluations left them
            const int xw = n * n + 2, xs = cache_x_slot(s, msp);
            for (int it = threadIdx.x; it < (nsec - 2) * xw; it += blockDim.x) {
              const int k = 1 + it / xw, w = it - (k - 1) * xw;
              cache_entry(s, cache, msp, wrap_slice(ifirst1 + k, M))[xs + w] =
                  m.xstage[(size_t)k * m.xstage_stride + w];
            }
          }
          __syncthreads();
          for (int k = 1 + threadIdx.x; k < nsec - 1; k += blockDim.x) {
            const int t1 = wrap_slice(ifirst1 + k, M);
            double* e = cache_entry(s, cache, msp, t1);
            e[1] = m.ndm[k];
            e[0] = (double)epoch[msp];
            double* o = cache_entry(s, cache, msp, (t1 + M / 2) % M);
            o[0] = NaN;
            const int ms = cache_mask_slot(s, msp);
            o[ms] = __longlong_as_double(__double_as_longlong(o[ms]) | (1ll << jcol));
          }
        }
      }
      if (threadIdx.x == 0 && rec) {
        rec->ifirst1 = ifirst1;
        rec->ifirst2 = ifirst2;
        rec->ipart = ipart;
        rec->reject_level = reject;
      }
      __syncthreads();
      // SerialPaths::putBeads / putDoubleBeads (src/base/SerialPaths.cc:143-205).
      // The sections come back unchanged but for the moving particle's interior
      // beads of section 1 when the move was accepted, so only those are
      // written, unless the two sections overlap beyond their end slices
      // (2^L > M/2), where pi-qmc's put order decides which copy a shared
      // slice keeps and both sections are written in that order.
      if (fixed && (1 << L) > M / 2) {
        if (ifirst1 < M / 2 - 1) {
          store_section(s, path, ifirst1, m.s1x, m.s1y, m.s1z);
          __syncthreads();
          store_section(s, path, ifirst2, m.s2x, m.s2y, m.s2z);
        } else {
          store_section(s, path, ifirst2, m.s2x, m.s2y, m.s2z);
          __syncthreads();
          store_section(s, path, ifirst1, m.s1x, m.s1y, m.s1z);
        }
      } else if (reject < 0) {
        for (int k = 1 + threadIdx.x; k < nsec - 1; k += blockDim.x) {
          const int islice = ifirst1 + k;
          if (islice < 0) continue;
          const int t = islice < M ? islice : islice % M;
          double* dst = path + ((size_t)t * np + ipart) * 3;
          dst[0] = m.s1x[k * np + ipart];
          dst[1] = m.s1y[k * np + ipart];
          dst[2] = m.s1z[k * np + ipart];
        }
      }
      __syncthreads();
    }
    if (threadIdx.x == 0) {
      P.state[r].attempt = att0 + (uint32_t)nat;
      P.state[r].status = status;
      P.state[r].accepted += nacc;
      P.state[r].attempted += nat;
      for (int k = 0; k < kMaxSpecies; ++k) {
        P.state[r].node_scale[k] = scale[k];
        P.state[r].epoch[k] = epoch[k];
      }
    }
    __syncthreads();
  }
}

}  // namespace pimc
