// Device-side data structures and physics for the bisection hot path.
// Each function cites the pi-qmc routine whose arithmetic it follows.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "pimc_rng.h"

namespace pimc {

constexpr int kMaxSpecies = 4;
constexpr int kMaxTables = 10;
constexpr int kMaxNs = 32;  // particles per node-model species
constexpr int kMaxLevels = 8;  // levels 0..nlevel+1
constexpr int kBlock = 256;     // threads of the estimator and entry-point kernels
constexpr int kMaxBlock = 512;  // largest section-kernel block (64..512 threads)
constexpr int kWarps = kMaxBlock / 32;  // reduction slots

struct DevTable {
  const double* ugrid;  // (ngpts,2,ndata)
  const float* ugrid32; // same table in FP32 (mixed precision)
  int ngpts, norder, ndata, s1, s2;
  int ifirst1, npart1, ifirst2, npart2;
  double rgridinv, logrratioinv;
};

struct DevSys {
  int npart, nspecies, nslice, nlevel, nsec;
  int spec_first[kMaxSpecies], spec_count[kMaxSpecies];
  double mass[kMaxSpecies], lambda[kMaxSpecies], charge[kMaxSpecies];
  double sho_omega[kMaxSpecies], prim_a[kMaxSpecies], prim_b[kMaxSpecies];
  int node_kind[kMaxSpecies];
  double node_c[kMaxSpecies], node_cosh[kMaxSpecies];  // SHONodes constants
  double node_dk[kMaxSpecies];  // sqrt(2 m / tau): nodal distance = node_dk / |grad ln det|
  // FreeParticleNodes: PeriodicGaussian(alpha = m T, L) per species and axis.
  double pg_nome[kMaxSpecies][3], pg_pref[kMaxSpecies][3], pg_k[kMaxSpecies][3];
  int pg_nmax[kMaxSpecies][3];
  double tau;
  // Per-level constants, evaluated on the host with the reference's expressions
  // (src/action/SpringAction.cc:72, src/advancer/mover/FreeMover.cc:78-79,
  // src/action/SHOAction.cc:31-36,77-82), so no thread repeats them.
  double spr_inv2s2[kMaxLevels][kMaxSpecies];
  double mov_sigma[kMaxLevels][kMaxSpecies], mov_inv2s2[kMaxLevels][kMaxSpecies];
  double sho_cosh[kMaxLevels][kMaxSpecies], sho_div1[kMaxLevels][kMaxSpecies];
  double sho_div2[kMaxLevels];
  double sho_coth[kMaxSpecies], sho_csch[kMaxSpecies], sho_cosh0[kMaxSpecies];
  // The mixed form's SHO link action without cancellation:
  // a |r1 - r0|^2 + b r0.r1, a = (m / 2 tau') (x coth x - 1), b = m w tanh(x / 2), x = w tau'
  float sho_a[kMaxLevels][kMaxSpecies], sho_b[kMaxLevels][kMaxSpecies];
  // Delayed rejection (MultiLevelSampler's delayedRejection): on, and the
  // second proposal's width and 1 / (2 width^2) at level nlevel - 1
  int dr;
  double dr_sigma[kMaxSpecies], dr_inv2s2[kMaxSpecies];
  double cell[3], cellb[3], rcut2;
  float rcut2_lo;  // the mixed form's FP32 pre-test of pbc (pbc_f): rcut2 (1 - 1e-5)
  int spring, coulomb, ewald, mover, fixed_node;
  int mixed;  // PIMC_PREC_MIXED: pair-action terms in FP32, accumulated in FP64
  double epsilon;
  int ntab;
  DevTable tab[kMaxTables];
  int totk;
  const int* kvec;
  const double* vk;
  double one_over_2v, self_energy, deltak[3];
  int ikmax[3];
  int ns_max;           // largest node-species count
  uint32_t stream_id;     // random stream of this replica (its replica or request id)
  long long nc_offset;    // doubles into the Slater-result cache pool (-1: no cache)
  int nc_stride;          // doubles per cache entry
  // Structure factors rho_k = sum_j q_j e^{ik.r_j} of every path slice, kept as
  // integers on a fixed-point grid so that incremental updates equal a fresh sum
  // bit for bit: [nslice][totk][re, im].
  long long ek_offset;    // int64 words into the structure-factor cache (-1: none)
  double ek_scale;        // grid spacing 1/ek_scale (a power of two)
  long long path_offset;  // doubles into the path pool
  long long inv_offset;   // doubles into the node scratch pool (-1: shared memory)
};

// Mutable per-replica state kept on the device between launches.
struct DevState {
  uint32_t attempt;
  uint32_t status;
  long long accepted;
  long long attempted;
  double node_scale[kMaxSpecies];
  int epoch[kMaxSpecies];  // bumped whenever a node model's scale changes
};

// ---------------------------------------------------------------- helpers

__device__ __forceinline__ double dot3(double ax, double ay, double az, double bx, double by,
                                       double bz) {
  // (a0 b0 + a1 b1) + a2 b2 without contraction, as blitz::dot evaluates it.
  return __dadd_rn(__dadd_rn(__dmul_rn(ax, bx), __dmul_rn(ay, by)), __dmul_rn(az, bz));
}

// SuperCell::pbc (src/util/SuperCell.cc:25-34): minimum image, only applied
// when |v|^2 exceeds a quarter of the shortest side squared.
__device__ __forceinline__ void pbc(const DevSys& s, double& x, double& y, double& z) {
  if (dot3(x, y, z, x, y, z) > s.rcut2) {
    const double ix = floor(__dadd_rn(__dmul_rn(s.cellb[0], x), 1000.5)) - 1000;
    const double iy = floor(__dadd_rn(__dmul_rn(s.cellb[1], y), 1000.5)) - 1000;
    const double iz = floor(__dadd_rn(__dmul_rn(s.cellb[2], z), 1000.5)) - 1000;
    x = __dsub_rn(x, __dmul_rn(s.cell[0], ix));
    y = __dsub_rn(y, __dmul_rn(s.cell[1], iy));
    z = __dsub_rn(z, __dmul_rn(s.cell[2], iz));
  }
}

// The mixed form's minimum image of an FP64 difference, rounded to FP32 for
// its FP32 terms: pbc()'s decision taken in FP32 first, against rcut2 less
// 1e-5 relative (the FP32 sum of three rounded squares errs by under 5e-7
// relative, all terms positive), so every vector pbc() would image passes
// the pre-test and then takes pbc()'s own FP64 test and image; the others
// skip its FP64 dot product.
__device__ __forceinline__ void pbc_f(const DevSys& s, double x, double y, double z, float& fx,
                                      float& fy, float& fz) {
  fx = (float)x;
  fy = (float)y;
  fz = (float)z;
  if (fx * fx + fy * fy + fz * fz > s.rcut2_lo) {
    pbc(s, x, y, z);
    fx = (float)x;
    fy = (float)y;
    fz = (float)z;
  }
}

// PeriodicGaussian::evaluate (src/util/PeriodicGaussian.cc:20-40): the theta
// series value pref (1 + 2 sum_n q^(n^2) cos(n k x)) and its gradient
// -2 pref k sum_n n q^(n^2) sin(n k x), n < nmax.  pi-qmc builds the terms by a
// complex recurrence (q^(2n-1) e^(ikx) per step); here cos(n k x) and
// sin(n k x) follow the Chebyshev recurrence t_(n+1) = 2 cos(kx) t_n - t_(n-1)
// and the weights q^(n^2) the product q^(n^2) q^(2n+1): seven FP64 operations
// a term instead of fourteen, the same sums to ~1e-13 relative where the
// series nearly cancels (far smaller elsewhere).  Rounded operations
// throughout: every call site computes the same bits.
__device__ __forceinline__ double pg_eval(double nome, double pref, double k, int nmax, double x,
                                          double* grad) {
  double sw, cw;
  sincos(__dmul_rn(k, x), &sw, &cw);
  const double c2 = __dmul_rn(2.0, cw), q2 = __dmul_rn(nome, nome);
  double cp = 1.0, cc = cw, sp = 0.0, sc = sw;  // cos, sin of (n - 1) k x and n k x
  double w = nome, step = nome;                  // q^(n^2), q^(2n - 1)
  double s0 = 0.0, s1 = 0.0;
  for (int n = 1; n < nmax; ++n) {
    s0 = __fma_rn(w, cc, s0);
    s1 = __fma_rn(__dmul_rn(double(n), w), sc, s1);
    step = __dmul_rn(step, q2);
    w = __dmul_rn(w, step);
    const double cn = __fma_rn(c2, cc, -cp), sn = __fma_rn(c2, sc, -sp);
    cp = cc;
    cc = cn;
    sp = sc;
    sc = sn;
  }
  *grad = __dmul_rn(__dmul_rn(__dmul_rn(pref, 2.0), -k), s1);
  return __dmul_rn(pref, __fma_rn(2.0, s0, 1.0));
}

// Pair-action table lookup on the logarithmic grid
// (PairAction::u00 / uk0 / uk0CalcDerivatives, src/action/PairAction.cc:601-655).
// The range tests come before the conversion to an integer and are written so
// that a NaN or infinite distance takes a clamped branch: converting NaN to int
// is not defined to give an in-range index.  For finite q >= 1 the branches
// are pi-qmc's (i = int(x) > ngpts - 2 exactly when x >= ngpts - 1).
__device__ __forceinline__ void tab_locate(const DevTable& t, double q, int& i, double& x) {
  q *= t.rgridinv;
  x = log(q) * t.logrratioinv;
  if (!(q >= 1)) {
    i = 0;
    x = 0;
  } else if (!(x < t.ngpts - 1)) {
    i = t.ngpts - 2;
    x = 1;
  } else {
    i = (int)x;
    x -= i;
  }
}

__device__ __forceinline__ double tab_u00(const DevTable& t, double r) {
  int i;
  double x;
  tab_locate(t, r, i, x);
  const double* g = t.ugrid + (size_t)i * 2 * t.ndata;
  return (1 - x) * __ldg(g) + x * __ldg(g + 2 * t.ndata);
}

__device__ __forceinline__ double tab_uk0(const DevTable& t, double q, double s2) {
  int i;
  double x;
  tab_locate(t, q, i, x);
  const double* g0 = t.ugrid + (size_t)i * 2 * t.ndata;
  const double* g1 = g0 + 2 * t.ndata;
  double a = 0;
  for (int k = t.norder; k >= 0; k--) a = a * s2 + ((1 - x) * __ldg(g0 + k) + x * __ldg(g1 + k));
  return a;
}

__device__ __forceinline__ void tab_uk0d(const DevTable& t, double q, double s2, double& u,
                                         double& ut) {
  int i;
  double x;
  tab_locate(t, q, i, x);
  const double* g0 = t.ugrid + (size_t)i * 2 * t.ndata;
  const double* g1 = g0 + 2 * t.ndata;
  u = 0;
  ut = 0;
  for (int k = t.norder; k >= 0; k--) {
    u = u * s2 + ((1 - x) * __ldg(g0 + k) + x * __ldg(g1 + k));
    ut = ut * s2 + ((1 - x) * __ldg(g0 + t.ndata + k) + x * __ldg(g1 + t.ndata + k));
  }
}

// FP32 variants for the mixed-precision form (same grid, FP32 coefficients).
__device__ __forceinline__ float tab_uk0_f(const DevTable& t, float q, float s2, int norder_eff) {
  q *= (float)t.rgridinv;
  float x = __logf(q) * (float)t.logrratioinv;
  int i;  // range tests before the conversion, as tab_locate
  if (!(q >= 1.f)) {
    i = 0;
    x = 0.f;
  } else if (!(x < (float)(t.ngpts - 1))) {
    i = t.ngpts - 2;
    x = 1.f;
  } else {
    i = (int)x;
    x -= i;
  }
  const float* g0 = t.ugrid32 + (size_t)i * 2 * t.ndata;
  const float* g1 = g0 + 2 * t.ndata;
  float a = 0.f;
  for (int k = norder_eff; k >= 0; k--) a = fmaf(a, s2, fmaf(x, __ldg(g1 + k) - __ldg(g0 + k), __ldg(g0 + k)));
  return a;
}

// FP32 tau derivative of the off-diagonal series (uk0CalcDerivatives' utau).
__device__ __forceinline__ float tab_uk0d_tau_f(const DevTable& t, float q, float s2) {
  q *= (float)t.rgridinv;
  float x = __logf(q) * (float)t.logrratioinv;
  int i;  // range tests before the conversion, as tab_locate
  if (!(q >= 1.f)) {
    i = 0;
    x = 0.f;
  } else if (!(x < (float)(t.ngpts - 1))) {
    i = t.ngpts - 2;
    x = 1.f;
  } else {
    i = (int)x;
    x -= i;
  }
  const float* g0 = t.ugrid32 + (size_t)i * 2 * t.ndata + t.ndata;
  const float* g1 = g0 + 2 * t.ndata;
  float a = 0.f;
  for (int k = t.norder; k >= 0; k--) a = fmaf(a, s2, fmaf(x, __ldg(g1 + k) - __ldg(g0 + k), __ldg(g0 + k)));
  return a;
}

// Error-free sum of two doubles (Knuth TwoSum) for compensated accumulation.
__device__ __forceinline__ void two_sum(double a, double b, double& s, double& e) {
  s = a + b;
  const double bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

// A compensated FP32 sum (Knuth's TwoSum per term, the rounding errors
// collected in a second float): the mixed form's sums over links and pairs.
struct FSum {
  float s = 0.f, c = 0.f;
  __device__ __forceinline__ void add(float t) {
    const float u = __fadd_rn(s, t);
    const float bb = __fsub_rn(u, s);
    c = __fadd_rn(c, __fadd_rn(__fsub_rn(s, __fsub_rn(u, bb)), __fsub_rn(t, bb)));
    s = u;
  }
  __device__ __forceinline__ double value() const { return (double)s + (double)c; }
};

// Deterministic block sum of one double per thread (fixed tree order).
__device__ __forceinline__ double block_sum(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
  if (nw == 1) return __shfl_sync(0xffffffffu, v, 0);
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  if (w == 0) {
    v = (l < nw) ? red[l] : 0.0;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (l == 0) red[kWarps] = v;
  }
  __syncthreads();
  return red[kWarps];
}

}  // namespace pimc
