// The bisection section-move kernel: one CTA advances one replica through a
// sequence of section-move attempts, entirely on the device.
//
// Per attempt (pi-qmc order: SectionChooser.cc:30-48, DoubleSectionChooser.cc:33-65):
//   SectionChooser::run / DoubleSectionChooser::run   -> choose section(s), stage in smem
//   FixedNodeAction::initialize                        -> det + distances on every slice
//   SimpleParticleChooser::chooseParticles             -> moving particle
//   MultiLevelSampler::tryMove / DoubleMLSampler::tryMove, levels L..0:
//       FreeMover(PBC)::makeMove, CompositeAction::getActionDifference,
//       FixedNodeAction::getActionDifference, Metropolis test
//   SerialPaths::putBeads / putDoubleBeads             -> section(s) back to HBM
//
// Random numbers come from the counter-addressed streams of pimc_rng.h, so the
// CPU checkers can replay exactly the numbers a replica consumed.
#pragma once
#include "pimc_device.cuh"

namespace pimc {

// Shared-memory working set of one CTA (carved from dynamic shared memory).
struct Smem {
  double *s1x, *s1y, *s1z;  // section 1: [nsec][npart]
  double *s2x, *s2y, *s2z;  // section 2 (fixed node)
  double *mx, *my, *mz;     // moving beads [nsec]
  double* red;              // reduction scratch
  double* vred;             // vector reductions: [8][kWarps] partials, then 8 sums
  double* dm;               // [nspecies][nsec] determinants at section set-up
  double* ndm;              // [nsec] determinants of the moving species' new slices
  double* dist;             // [nsec][2][ns_max] distances at set-up (moving species)
  double* ndist;            // [nsec][2][ns_max] distances of the new path
  double* ewt;              // Ewald exp(ik.r) tables: [kx, ky, kz rows][ewt_cols]
  double* qpart;            // [npart] charges
  int* ictl;                // control words
  double* nodescr;          // per-warp node scratch (smem or global)
  double* ecache;           // [nsec][n*n] exp matrices of the moving species (SHONodes)
  double* ncol;             // [nsec][ncol_stride] recomputed column of each changed slice
  int ncol_stride;          // ns_max (SHO exp column) or 4 ns_max (free-particle values + gradients)
  double* nrm;              // [2^L - 1][3] the attempt's proposal normals
  int nodescr_stride;       // doubles per warp
  double* nodecold;         // cold parts of the node scratch when apart (global), or null
  int nodecold_stride;      // doubles per warp
  int ewt_cols;             // bead columns of the Ewald tables area
  double* xstage;           // mixed form: [nsec][xstage_stride] inverse blocks (global), or null
  int xstage_stride;
};


enum {
  C_IFIRST1 = 0, C_IFIRST2, C_IPART, C_REJECT, C_FLAG, C_SCANK, C_ERRS, C_NMISS, C_NCTL = 16
};

struct SectionSizes {
  // all counts in doubles
  static __host__ __device__ long long section(int nsec, int npart) { return 3LL * nsec * npart; }
};

// Positions of particle p on section slice t, with the moving bead substituted.
struct SliceView {
  const double *sx, *sy, *sz;
  int npart;
  int t;
  int imov;  // substituted particle or -1
  double mxv, myv, mzv;
  __device__ __forceinline__ void get(int p, double& x, double& y, double& z) const {
    if (p == imov) {
      x = mxv;
      y = myv;
      z = mzv;
    } else {
      const int o = t * npart + p;
      x = sx[o];
      y = sy[o];
      z = sz[o];
    }
  }
};

// ------------------------------------------------------------------ node model
// The mixed form's Sherman-Morrison updates of cached inverses: at most
// kSmRefresh updates between two factorisations of a slice pair's matrix, and
// none whose determinant ratio is below kSmMinRatio in magnitude.
// A factorisation whose conditioning estimate n max|a| max|inv| exceeds
// kSmMaxCond starts no updates: an update's relative error grows with the
// condition number (the SHONodes matrices of a cold dot reach 1e13 and more).
constexpr double kSmRefresh = 16.0;
constexpr double kSmMinRatio = 0.05;
constexpr double kSmMaxCond = 1e7;
// Scratch doubles one lane group needs for an n-particle species: a hot part
// (the LU and the inverse, rewritten at every elimination step, and the
// reciprocal pivots) and a cold part (the SHO exp matrix, or the free-particle
// gradient matrices: written once, read once).
__host__ __device__ constexpr int node_group_hot(int n) { return 2 * n * n + n + 1; }
__host__ __device__ constexpr int node_group_cold(int n, bool free_nodes = true) {
  return n * n + (free_nodes ? 3 * n * n : 0);
}
__host__ __device__ constexpr int node_group_scratch(int n, bool free_nodes = true) {
  return node_group_hot(n) + node_group_cold(n, free_nodes);
}

// Slater scratch of lane group g of a warp: the hot part (with the cold part
// after it, unless the layout keeps cold parts apart) and the cold part.
__device__ __forceinline__ double* group_scr(const Smem& m, int warp, int g, int n, bool free_nodes) {
  return m.nodescr + (size_t)warp * m.nodescr_stride +
         g * (m.nodecold ? node_group_hot(n) : node_group_scratch(n, free_nodes));
}
__device__ __forceinline__ double* group_cold(const Smem& m, int warp, int g, int n, bool free_nodes) {
  return m.nodecold ? m.nodecold + (size_t)warp * m.nodecold_stride + g * node_group_cold(n, free_nodes)
                    : nullptr;
}

// NodeModel::evaluate (+ evaluateDistance) for one species on one slice pair,
// executed by a group of W lanes (W = 8, 16 or 32; 32/W groups per warp each
// take their own slice pair).  Lanes own matrix rows.  LU with partial pivoting
// (first largest |pivot|, LAPACK dgetrf semantics), determinant from the U
// diagonal and pivots, inverse by solving A X = I column per lane (dgetri
// semantics), then the log-gradient nodal distances
// (src/fixednode/SHONodes.cc:51-170, src/fixednode/FreeParticleNodes.cc:72-234).
// full = 0: determinant only.  Every lane of the warp must call this (the
// shuffles span the warp); a group with write = false computes but stores
// nothing.  For SHONodes, ecache (n*n, or null) holds the slice's exp matrix:
// jcol < 0 fills it, jcol >= 0 reuses it and recomputes column jcol only (the
// other columns' inputs are unchanged, so the values are bit-identical).
// kSm: the variant with the mixed form's Sherman-Morrison updates and inverse
// blocks (xin / xout); without it those arguments are ignored and the
// evaluation is the plain factorisation.
template <int W, bool kSm = false>
static __device__ __noinline__ void node_eval_group(const DevSys& s, int sp, const SliceView& v1,
                                const SliceView& v2, double scale, double* scr, int full,
                                double* ecache, int jcol, bool write, double& det_out,
                                int& err_out, double* d1, double* d2,
                                double* newcol = nullptr, unsigned rowmask = 0xffffffffu,
                                double* cold = nullptr, const double* xin = nullptr,
                                double det_in = 0.0, double* xout = nullptr,
                                double xepoch = 0.0) {
  constexpr unsigned FULL = 0xffffffffu;
  const int gl = threadIdx.x & (W - 1);
  const int n = s.spec_count[sp];
  const int f = s.spec_first[sp];
  // hot part at scr; the cold part follows it unless given apart
  double* A = scr;          // n*n column-major, LU; after the inverse: the distance weights
  double* X = A + n * n;    // n*n inverse, column-major
  double* R = X + n * n;    // n reciprocals of the U diagonal
  double* E = cold ? cold : scr + node_group_hot(n);  // n*n exp values (SHO nodes)
  double* G = E + n * n;    // 3 n*n gradient factors (free-particle nodes)
  const bool sho = s.node_kind[sp] == 1;
  // --- build the Slater matrix: A(i,j) = scale * rho(r1_j, r2_i)
  // Elements come from ecache where it holds them (a column update keeps every
  // column but jcol; a row refresh keeps the rows outside rowmask); the others
  // are computed.  Whole rows (all of them without a cache, the stale ones on a
  // refresh) go one element per lane and step, so that refreshing one or two
  // rows still spreads over the group; the new column of a column update goes
  // one row per lane.  Every element is the same rounded arithmetic wherever
  // it is computed, so cached and recomputed values agree bit for bit.
  const int nn = n * n;
  const unsigned nmask = n >= 32 ? 0xffffffffu : ((1u << n) - 1u);
  const unsigned rows_new = !ecache ? nmask : (jcol < 0 ? (rowmask & nmask) : 0u);
  // element (i, j): value into A (scaled), E (SHO) or G (gradients), and into
  // ecache (a refresh) or newcol (the new column) when this group writes
  auto element = [&](int i, int j) {
    double rix, riy, riz, rjx, rjy, rjz;
    v2.get(f + i, rix, riy, riz);
    v1.get(f + j, rjx, rjy, rjz);
    const bool to_cache = ecache && jcol < 0 && write;
    const bool to_col = newcol && j == jcol && write;
    if (sho) {
      const double ri2 = dot3(rix, riy, riz, rix, riy, riz);
      const double rj2 = dot3(rjx, rjy, rjz, rjx, rjy, rjz);
      const double rirj = dot3(rix, riy, riz, rjx, rjy, rjz);
      const double q = __dsub_rn(__dmul_rn(__dadd_rn(ri2, rj2), s.node_cosh[sp]),
                                 __dmul_rn(2.0, rirj));
      const double e = exp(__dmul_rn(-s.node_c[sp], q));
      if (to_cache) ecache[j * n + i] = e;
      if (to_col) newcol[i] = e;
      E[j * n + i] = e;
      A[j * n + i] = scale * e;
    } else {
      double dx = rjx - rix, dy = rjy - riy, dz = rjz - riz;
      pbc(s, dx, dy, dz);
      double g0, g1, g2;
      const double v0 = pg_eval(s.pg_nome[sp][0], s.pg_pref[sp][0], s.pg_k[sp][0], s.pg_nmax[sp][0], dx, &g0);
      const double v1v = pg_eval(s.pg_nome[sp][1], s.pg_pref[sp][1], s.pg_k[sp][1], s.pg_nmax[sp][1], dy, &g1);
      const double v2v = pg_eval(s.pg_nome[sp][2], s.pg_pref[sp][2], s.pg_k[sp][2], s.pg_nmax[sp][2], dz, &g2);
      const double val = v0 * v1v * v2v;
      double gx = g0 / (v0 + 1e-300), gy = g1 / (v1v + 1e-300), gz = g2 / (v2v + 1e-300);
      gx *= v0; gy *= v0; gz *= v0;
      gx *= v1v; gy *= v1v; gz *= v1v;
      gx *= v2v; gy *= v2v; gz *= v2v;
      if (to_cache) {
        ecache[j * n + i] = val;
        ecache[nn + j * n + i] = gx;
        ecache[2 * nn + j * n + i] = gy;
        ecache[3 * nn + j * n + i] = gz;
      }
      if (to_col) {
        newcol[i] = val;
        newcol[n + i] = gx;
        newcol[2 * n + i] = gy;
        newcol[3 * n + i] = gz;
      }
      A[j * n + i] = scale * val;
      G[j * n + i] = gx;
      G[nn + j * n + i] = gy;
      G[2 * nn + j * n + i] = gz;
    }
  };
  // cached rows (with the new column of a column update), one row per lane
  if (ecache && gl < n && !((rows_new >> gl) & 1u)) {
    const int i = gl;
    for (int j = 0; j < n; ++j) {
      if (jcol >= 0 && j == jcol) {
        element(i, j);
      } else if (sho) {
        const double e = ecache[j * n + i];
        E[j * n + i] = e;
        A[j * n + i] = scale * e;
      } else {
        A[j * n + i] = scale * ecache[j * n + i];
        G[j * n + i] = ecache[nn + j * n + i];
        G[nn + j * n + i] = ecache[2 * nn + j * n + i];
        G[2 * nn + j * n + i] = ecache[3 * nn + j * n + i];
      }
    }
  }
  // rows computed in full, one element per lane and step
  const int nrows = __popc(rows_new);
  for (int e = gl; e < nrows * n; e += W) {
    unsigned rm = rows_new;
    for (int q = e / n; q > 0; --q) rm &= rm - 1u;  // drop the first e/n set rows
    element(__ffs(rm) - 1, e % n);
  }
  __syncwarp();
  int info = 0;
  // --- the mixed form: Sherman-Morrison updates of the cached inverse (xin:
  // its [epoch, updates, inverse] block) instead of a factorisation, for the
  // new column jcol of a level evaluation or each changed row of a refresh.
  // A group updates when its block is of the current scale (epoch), has had
  // fewer than kSmRefresh updates since its last factorisation, and every
  // determinant ratio is at least kSmMinRatio in magnitude (a refresh: at most
  // n/2 rows); otherwise, or when another writing group of the warp cannot,
  // the warp factorises as below.  Every lane takes part in the shuffles.
  bool use_sm = false;
  bool good = kSm && xin != nullptr && xin[0] == xepoch && xin[1] < kSmRefresh;
  // (a warp none of whose writing groups can update factorises at once)
  if (kSm && __any_sync(FULL, good && write) && __all_sync(FULL, good || !write)) {
    const double* xc = good ? xin + 2 : nullptr;
    for (int k = gl; k < nn; k += W) X[k] = xc ? xc[k] : 0.0;
    __syncwarp();
    double det = det_in;
    if (jcol >= 0) {
      // column jcol replaced by u = A(:, jcol): w = inv u, ratio = w_jcol,
      // inv'(a, b) = inv(a, b) - (w_a - [a = jcol]) inv(jcol, b) / ratio
      double w = 0.0;
      if (gl < n)
        for (int i = 0; i < n; ++i) w = __fma_rn(X[i * n + gl], A[jcol * n + i], w);
      const double ratio = __shfl_sync(FULL, w, jcol, W);
      good = good && fabs(ratio) >= kSmMinRatio;
      use_sm = __all_sync(FULL, good || !write);
      if (use_sm) {
        const double rj = gl < n ? X[gl * n + jcol] : 0.0;  // inv(jcol, b), b = gl
        const double f = gl < n ? (w - (gl == jcol ? 1.0 : 0.0)) / ratio : 0.0;
        __syncwarp();
        for (int e0 = 0; e0 < nn; e0 += W) {
          const int e = e0 + gl;
          const bool on = e < nn;
          const int b = on ? e / n : 0, a = on ? e - b * n : 0;
          const double fa = __shfl_sync(FULL, f, a, W);
          const double rb = __shfl_sync(FULL, rj, b, W);
          if (on) X[b * n + a] = __fma_rn(-fa, rb, X[b * n + a]);
        }
        det = __dmul_rn(det_in, ratio);
      }
    } else {
      // each changed row i in turn, v = A(i, :): z = v inv, ratio = z_i,
      // inv'(a, b) = inv(a, b) - inv(a, i) (z_b - [b = i]) / ratio
      const int nr = __popc(rows_new);
      good = good && nr > 0 && 2 * nr <= n;
      const unsigned nrmax = __reduce_max_sync(FULL, good ? (unsigned)nr : 0u);
      unsigned rm = good ? rows_new : 0u;
      for (unsigned k = 0; k < nrmax; ++k) {
        const bool live = rm != 0u;
        const int i = live ? __ffs(rm) - 1 : 0;
        rm &= rm - 1u;
        double z = 0.0;
        if (gl < n)
          for (int j = 0; j < n; ++j) z = __fma_rn(A[j * n + i], X[gl * n + j], z);
        const double ratio = __shfl_sync(FULL, z, i, W);
        const double ci = gl < n ? X[i * n + gl] : 0.0;  // inv(a, i), a = gl
        const double g = gl < n ? (z - (gl == i ? 1.0 : 0.0)) / ratio : 0.0;
        __syncwarp();
        for (int e0 = 0; e0 < nn; e0 += W) {
          const int e = e0 + gl;
          const bool on = e < nn && live;
          const int b = e < nn ? e / n : 0, a = e < nn ? e - b * n : 0;
          const double ca = __shfl_sync(FULL, ci, a, W);
          const double gb = __shfl_sync(FULL, g, b, W);
          if (on) X[b * n + a] = __fma_rn(-ca, gb, X[b * n + a]);
        }
        __syncwarp();
        if (live) {
          det = __dmul_rn(det, ratio);
          good = good && fabs(ratio) >= kSmMinRatio;
        }
      }
      use_sm = __all_sync(FULL, good || !write);
    }
    if (use_sm && write) {
      det_out = det;
      err_out = 0;
    }
  }
  double amax = 0.0;  // max |a| of the matrix, for the conditioning estimate (mixed form)
  // every lane takes part in the shuffles
  const bool xany = kSm && __any_sync(FULL, xout != nullptr);
  if (!use_sm) {
  if (xany) {
    for (int k = gl; k < nn; k += W) amax = fmax(amax, fabs(A[k]));
#pragma unroll
    for (int o = W / 2; o > 0; o >>= 1) amax = fmax(amax, __shfl_xor_sync(FULL, amax, o, W));
  }
  // --- LU with partial pivoting (the pivot is the first largest |a|)
  unsigned pivbits = 0;  // bit j set: row j was interchanged
  int piv_lane = gl;     // piv[gl] for gl < n
  for (int j = 0; j < n; ++j) {
    // |a| compared through its bit pattern (monotonic for non-negative
    // doubles), so the search runs on the integer pipe; -1 marks idle lanes
    long long av = (gl >= j && gl < n)
                       ? (__double_as_longlong(A[j * n + gl]) & 0x7fffffffffffffffLL)
                       : -1LL;
    int ai = gl;
#pragma unroll
    for (int o = W / 2; o > 0; o >>= 1) {
      const long long ov = __shfl_down_sync(FULL, av, o, W);
      const int oi = __shfl_down_sync(FULL, ai, o, W);
      if (ov > av || (ov == av && oi < ai)) {
        av = ov;
        ai = oi;
      }
    }
    const int p = __shfl_sync(FULL, ai, 0, W);
    if (gl == j) piv_lane = p;
    const double apj = A[j * n + p];
    if (__double_as_longlong(apj) & 0x7fffffffffffffffLL) {  // apj != 0, on the integer pipe
      if (p != j) {
        pivbits |= 1u << j;
        for (int k = gl; k < n; k += W) {
          const double t = A[k * n + j];
          A[k * n + j] = A[k * n + p];
          A[k * n + p] = t;
        }
      }
      __syncwarp();
      const double rinv = __drcp_rn(A[j * n + j]);  // 1 / a, correctly rounded
      if (gl == j) R[j] = rinv;
      if (gl > j && gl < n) A[j * n + gl] *= rinv;
    } else if (info == 0) {
      info = j + 1;
    }
    __syncwarp();
    // trailing update, one element per lane and step: a(i,k) -= l(i,j) u(j,k)
    const int m = n - j - 1;
    if (m > 0) {
      int kk = gl / m, ii = gl - kk * m;
      const int dk = W / m, di = W - dk * m;
      for (int e = gl; e < m * m; e += W) {
        const int row = j + 1 + ii, col = j + 1 + kk;
        A[col * n + row] -= A[j * n + row] * A[col * n + j];
        ii += di;
        kk += dk;
        if (ii >= m) {
          ii -= m;
          ++kk;
        }
      }
    }
    __syncwarp();
  }
  // --- determinant (sequential product, as the reference)
  double det = 1.0;
  for (int i = 0; i < n; ++i) {
    det *= A[i * n + i];
    // times -1 for an interchanged row: a sign flip, exactly that product
    if ((pivbits >> i) & 1u) det = __longlong_as_double(__double_as_longlong(det) ^ (1LL << 63));
  }
  if (write) {
    det_out = det;
    err_out = info != 0;
  }
  if (!full) return;  // the same for every group of the warp
  // --- inverse: lane c solves A x = e_c
  int pos = gl;  // e_c after the row interchanges (every lane takes part in the shuffles)
  for (int j = 0; j < n; ++j) {
    const int pj = __shfl_sync(FULL, piv_lane, j, W);
    if (pos == j)
      pos = pj;
    else if (pos == pj)
      pos = j;
  }
  // Column c of X starts as e_pos(c); the substitutions then run one element
  // (column, row) per lane and step.  Every element receives the same FMAs in
  // the same order as a per-column solve, so the result is that solve's, bit
  // for bit: the forward steps before pos(c) would only subtract exact zeros
  // from zeros, and are skipped.
  const bool inv_ok = info == 0;
  if (inv_ok && gl < n)
    for (int i = 0; i < n; ++i) X[gl * n + i] = (i == pos) ? 1.0 : 0.0;
  int ordc = 0;  // the column whose unit vector sits at row gl
  for (int c = 0; c < n; ++c)
    if (__shfl_sync(FULL, pos, c, W) == gl) ordc = c;
  __syncwarp();
  for (int j = 0; j < n - 1; ++j) {  // forward: x(i) -= l(i,j) x(j), i > j
    // the columns nonzero at row j: order[q] for q <= j, rows j+1 .. n-1
    const int m = n - j - 1, cnt = (j + 1) * m;
    int q = gl / m, ii = gl - q * m;  // element e = gl + k W: (q, row j + 1 + ii)
    const int dq = W / m, di = W - dq * m;
    for (int e0 = 0; e0 < cnt; e0 += W) {
      const bool on = e0 + gl < cnt;
      const int c = __shfl_sync(FULL, ordc, on ? q : 0, W);
      if (inv_ok && on) {
        const int i = j + 1 + ii;
        X[c * n + i] -= A[j * n + i] * X[c * n + j];
      }
      ii += di;
      q += dq;
      if (ii >= m) {
        ii -= m;
        ++q;
      }
    }
    __syncwarp();
  }
  for (int j = n - 1; j >= 0; --j) {  // back: x(j) *= 1/u(j,j); x(i) -= u(i,j) x(j), i < j
    if (inv_ok)
      for (int c = gl; c < n; c += W) X[c * n + j] *= R[j];
    __syncwarp();
    if (inv_ok && j > 0) {
      int c = gl / j, ii = gl - c * j;
      const int dc = W / j, di = W - dc * j;
      for (int e = gl; e < n * j; e += W) {
        X[c * n + ii] -= A[j * n + ii] * X[c * n + j];
        ii += di;
        c += dc;
        if (ii >= j) {
          ii -= j;
          ++c;
        }
      }
    }
    __syncwarp();
  }
  }  // factorisation
  // the inverse and its update count for the cache (mixed form); a fresh
  // factorisation that is too ill-conditioned is marked as used up
  if (xany) {
    double xmax = 0.0;
    if (!use_sm) {
      for (int k = gl; k < nn; k += W) xmax = fmax(xmax, fabs(X[k]));
#pragma unroll
      for (int o = W / 2; o > 0; o >>= 1) xmax = fmax(xmax, __shfl_xor_sync(FULL, xmax, o, W));
    }
    if (write && xout) {
      for (int k = gl; k < nn; k += W) xout[2 + k] = X[k];
      if (gl == 0) {
        xout[0] = info == 0 ? xepoch : __longlong_as_double(0x7ff8000000000000LL);
        xout[1] = use_sm ? xin[1] + 1.0
                         : (n * amax * xmax <= kSmMaxCond ? 0.0 : kSmRefresh);
      }
    }
  }
  // --- nodal distances: d = sqrt(2m / (tau |grad ln det|^2)), the gradient
  // with respect to r1_j (d1) and r2_i (d2); inv(j,i) = X[i*n + j].  (No early
  // exit: a singular group simply skips them, so the warp stays converged.)
  const double dk = s.node_dk[sp];
  const bool ok = info == 0;
  if (sho) {
    // weights w(i,j) = inv(j,i) rho(i,j), shared by both gradients
    if (ok) {
      int j = gl / n, i = gl - j * n;
      const int dj = W / n, di = W - dj * n;
      for (int e = gl; e < n * n; e += W) {
        A[j * n + i] = X[i * n + j] * E[j * n + i];
        i += di;
        j += dj;
        if (i >= n) {
          i -= n;
          ++j;
        }
      }
    }
    __syncwarp();
    const double c = s.node_c[sp], ch = s.node_cosh[sp];
    const double fac = 2 * c * scale;
    // sum_i w(i,j) (r2_i - ch r1_j) = S - ch r1_j T with S = sum_i w(i,j) r2_i and
    // T = sum_i w(i,j): four FP64 operations a term instead of six
    if (ok && gl < n) {
      const int j = gl;  // d1: sum_i w(i,j) 2c (r2_i - ch r1_j)
      double rjx, rjy, rjz;
      v1.get(f + j, rjx, rjy, rjz);
      double sx = 0, sy = 0, sz = 0, tw = 0;
      for (int i = 0; i < n; ++i) {
        double rix, riy, riz;
        v2.get(f + i, rix, riy, riz);
        const double w = A[j * n + i];
        sx += w * rix;
        sy += w * riy;
        sz += w * riz;
        tw += w;
      }
      const double ct = ch * tw;
      const double lx = fac * (sx - ct * rjx), ly = fac * (sy - ct * rjy), lz = fac * (sz - ct * rjz);
      if (write) d1[j] = dk * rsqrt(dot3(lx, ly, lz, lx, ly, lz) + 1e-15);
    }
    if (ok && gl < n) {
      const int i = gl;  // d2: sum_j w(i,j) 2c (r1_j - ch r2_i)
      double rix, riy, riz;
      v2.get(f + i, rix, riy, riz);
      double sx = 0, sy = 0, sz = 0, tw = 0;
      for (int j = 0; j < n; ++j) {
        double rjx, rjy, rjz;
        v1.get(f + j, rjx, rjy, rjz);
        const double w = A[j * n + i];
        sx += w * rjx;
        sy += w * rjy;
        sz += w * rjz;
        tw += w;
      }
      const double ct = ch * tw;
      const double lx = fac * (sx - ct * rix), ly = fac * (sy - ct * riy), lz = fac * (sz - ct * riz);
      if (write) d2[i] = dk * rsqrt(dot3(lx, ly, lz, lx, ly, lz) + 1e-15);
    }
  } else {
    const double* Gx = G;
    const double* Gy = G + n * n;
    const double* Gz = G + 2 * n * n;
    if (ok && gl < n) {
      const int j = gl;  // d1: sum_i inv(j,i) dA(i,j)/dr1_j
      double lx = 0, ly = 0, lz = 0;
      for (int i = 0; i < n; ++i) {
        const double w = X[i * n + j];
        lx += w * Gx[j * n + i];
        ly += w * Gy[j * n + i];
        lz += w * Gz[j * n + i];
      }
      lx *= scale;
      ly *= scale;
      lz *= scale;
      if (write) d1[j] = dk * rsqrt(dot3(lx, ly, lz, lx, ly, lz) + 1e-15);
    }
    if (ok && gl < n) {
      const int i = gl;  // d2: sum_j inv(j,i) dA(i,j)/dr2_i, dA/dr2_i = -dA/dr1_j
      double lx = 0, ly = 0, lz = 0;
      for (int j = 0; j < n; ++j) {
        const double w = X[i * n + j];
        lx += w * Gx[j * n + i];
        ly += w * Gy[j * n + i];
        lz += w * Gz[j * n + i];
      }
      lx *= scale;
      ly *= scale;
      lz *= scale;
      if (write) d2[i] = dk * rsqrt(dot3(lx, ly, lz, lx, ly, lz) + 1e-15);
    }
  }
  __syncwarp();
}


// Group width for an n-particle species.
__host__ __device__ __forceinline__ int node_group_width(int n) {
  return n <= 8 ? 8 : (n <= 16 ? 16 : 32);
}

// One warp evaluates one slice pair (the entry-point kernels).
static __device__ void node_eval_warp(const DevSys& s, int sp, const SliceView& v1, const SliceView& v2,
                               double scale, double* scr, int full, double& det_out,
                               int& err_out, double* d1, double* d2) {
  node_eval_group<32>(s, sp, v1, v2, scale, scr, full, nullptr, -1, true, det_out, err_out, d1,
                      d2);
}

// ------------------------------------------------------------------ actions
// Per-thread partial of CompositeAction::getActionDifference for one moving
// particle ipart at one level: SpringAction (src/action/SpringAction.cc:56-98),
// SHOAction (src/action/SHOAction.cc:19-65), PrimSHOAction
// (src/action/PrimSHOAction.cc:21-58), PairAction per species pair
// (src/action/PairAction.cc:219-360).  Work items are links and (partner, link)
// pairs; each item contributes (new - old).
static __device__ __noinline__ double action_partial_mixed(const DevSys& s, const Smem& m,
                                                          int ipart, int level, int tid,
                                                          int nthreads);

static __device__ __noinline__ double action_partial(const DevSys& s, const Smem& m, int ipart, int level,
                                        int tid, int nthreads) {
  if (s.mixed) return action_partial_mixed(s, m, ipart, level, tid, nthreads);
  const int L = s.nlevel, np = s.npart;
  const int nStride = 1 << level;
  const int nlinks = 1 << (L - level);
  const int sp = [&] {
    int r = 0;
    for (int k = 0; k < s.nspecies; ++k)
      if (ipart >= s.spec_first[k] && ipart < s.spec_first[k] + s.spec_count[k]) r = k;
    return r;
  }();
  double acc = 0.0;
  // spring + SHO + PrimSHO: one item per link k (slices (k-1)*nStride, k*nStride)
  const double inv2Sigma2 = s.spr_inv2s2[level][sp];
  const double om = s.sho_omega[sp];
  const double coshwt = s.sho_cosh[level][sp], div1 = s.sho_div1[level][sp];
  const double div2 = s.sho_div2[level], msho = s.mass[sp];
  const bool prim = s.prim_a[sp] != 0 || s.prim_b[sp] != 0;
  // Pair tables the moving particle takes part in, and their partner ranges.
  int tb[kMaxTables], tjb[kMaxTables], tn[kMaxTables], nt = 0;
  if (s.coulomb) {
    for (int ti = 0; ti < s.ntab; ++ti) {
      const DevTable& t = s.tab[ti];
      if (ipart >= t.ifirst1 && ipart < t.ifirst1 + t.npart1) {
        tb[nt] = ti;
        tjb[nt] = t.ifirst2;
        tn[nt++] = t.npart2;
      } else if (ipart >= t.ifirst2 && ipart < t.ifirst2 + t.npart2) {
        tb[nt] = ti;
        tjb[nt] = t.ifirst1;
        tn[nt++] = t.npart1;
      }
    }
  }
  int total = nlinks;
  for (int q = 0; q < nt; ++q) total += tn[q] * nlinks;
  for (int item = tid; item < total; item += nthreads) {
    if (item < nlinks) {
      const int k = item + 1;
      const int t1 = k * nStride, t0 = t1 - nStride;
      const double n1x = m.mx[t1], n1y = m.my[t1], n1z = m.mz[t1];
      const double n0x = m.mx[t0], n0y = m.my[t0], n0z = m.mz[t0];
      const double o1x = m.s1x[t1 * np + ipart], o1y = m.s1y[t1 * np + ipart], o1z = m.s1z[t1 * np + ipart];
      const double o0x = m.s1x[t0 * np + ipart], o0y = m.s1y[t0 * np + ipart], o0z = m.s1z[t0 * np + ipart];
      if (s.spring) {
        double dx = n1x - n0x, dy = n1y - n0y, dz = n1z - n0z;
        pbc(s, dx, dy, dz);
        double ex = o1x - o0x, ey = o1y - o0y, ez = o1z - o0z;
        pbc(s, ex, ey, ez);
        const double nw = dx * dx * inv2Sigma2 + dy * dy * inv2Sigma2 + dz * dz * inv2Sigma2;
        const double od = ex * ex * inv2Sigma2 + ey * ey * inv2Sigma2 + ez * ez * inv2Sigma2;
        acc += nw - od;
      }
      if (om > 0) {
        double r0r0 = n0x * n0x + n0y * n0y + n0z * n0z;
        double r1r1 = n1x * n1x + n1y * n1y + n1z * n1z;
        double r0r1 = n0x * n1x + n0y * n1y + n0z * n1z;
        double dx = n1x - n0x, dy = n1y - n0y, dz = n1z - n0z;
        double d2 = dx * dx + dy * dy + dz * dz;
        const double nw = msho * om * ((r1r1 + r0r0) * coshwt - 2.0 * r0r1) * div1 - msho * d2 * div2;
        r0r0 = o0x * o0x + o0y * o0y + o0z * o0z;
        r1r1 = o1x * o1x + o1y * o1y + o1z * o1z;
        r0r1 = o0x * o1x + o0y * o1y + o0z * o1z;
        dx = o1x - o0x;
        dy = o1y - o0y;
        dz = o1z - o0z;
        d2 = dx * dx + dy * dy + dz * dz;
        const double od = msho * om * ((r1r1 + r0r0) * coshwt - 2.0 * r0r1) * div1 - msho * d2 * div2;
        acc += nw - od;
      }
      if (prim && k < nlinks) {
        double x = n1x, y = n1y, z = n1z;
        pbc(s, x, y, z);
        double x2 = x * x + y * y + z * z;
        const double kt = s.tau * nStride;
        const double nw = (s.prim_a[sp] * x2 + s.prim_b[sp] * x2 * x2) * kt;
        x = o1x;
        y = o1y;
        z = o1z;
        pbc(s, x, y, z);
        x2 = x * x + y * y + z * z;
        acc += nw - (s.prim_a[sp] * x2 + s.prim_b[sp] * x2 * x2) * kt;
      }
      continue;
    }
    int it = item - nlinks, q = 0;
    while (it >= tn[q] * nlinks) {
      it -= tn[q] * nlinks;
      ++q;
    }
    const DevTable& t = s.tab[tb[q]];
    const int jj = it / nlinks;
    const int j = tjb[q] + jj;
    if (j == ipart) continue;
    const int k = it - jj * nlinks + 1;
    const int t1 = k * nStride, t0 = t1 - nStride;
    const double pjx1 = m.s1x[t1 * np + j], pjy1 = m.s1y[t1 * np + j], pjz1 = m.s1z[t1 * np + j];
    const double pjx0 = m.s1x[t0 * np + j], pjy0 = m.s1y[t0 * np + j], pjz0 = m.s1z[t0 * np + j];
    const bool offdiag = level < 3 && t.norder > 0;
    double act[2];
#pragma unroll
    for (int pass = 0; pass < 2; ++pass) {
      double ax, ay, az, bx, by, bz;
      if (pass == 0) {
        ax = m.mx[t1]; ay = m.my[t1]; az = m.mz[t1];
        bx = m.mx[t0]; by = m.my[t0]; bz = m.mz[t0];
      } else {
        ax = m.s1x[t1 * np + ipart]; ay = m.s1y[t1 * np + ipart]; az = m.s1z[t1 * np + ipart];
        bx = m.s1x[t0 * np + ipart]; by = m.s1y[t0 * np + ipart]; bz = m.s1z[t0 * np + ipart];
      }
      double dx = ax - pjx1, dy = ay - pjy1, dz = az - pjz1;
      pbc(s, dx, dy, dz);
      double px = bx - pjx0, py = by - pjy0, pz = bz - pjz0;
      pbc(s, px, py, pz);
      const double r = sqrt(dot3(dx, dy, dz, dx, dy, dz));
      const double rp = sqrt(dot3(px, py, pz, px, py, pz));
      const double qq = 0.5 * (r + rp);
      double a;
      if (offdiag) {
        const double sx = dx - px, sy = dy - py, sz = dz - pz;
        const double s2 = dot3(sx, sy, sz, sx, sy, sz) / (qq * qq);
        a = tab_uk0(t, qq, s2) * nStride;
      } else {
        a = tab_u00(t, qq) * nStride;
      }
      act[pass] = a;
    }
    acc += act[0] - act[1];
  }
  return acc;
}

// The mixed form of action_partial: every term in FP32, the per-thread sum
// compensated (FSum) and returned in FP64 for the block reduction.  Spring:
// (|d_new|^2 - |d_old|^2) / (4 lambda tau'); SHO: a (|d_new|^2 - |d_old|^2) +
// b (r0.r1_new - r0.r1_old), the harmonic link action minus its free part
// rearranged so that nothing cancels (sho_a, sho_b); PrimSHO: (a x^2 + b x^4)
// tau' at the moved bead; pairs: PairAction's u00 / uk0 series on the FP32 copy
// of the table.  Differences of positions are formed (and minimum-imaged) in
// FP64 before they are rounded to FP32.
static __device__ __noinline__ double action_partial_mixed(const DevSys& s, const Smem& m,
                                                          int ipart, int level, int tid,
                                                          int nthreads) {
  const int L = s.nlevel, np = s.npart;
  const int nStride = 1 << level;
  const int nlinks = 1 << (L - level);
  int sp = 0;
  for (int k = 0; k < s.nspecies; ++k)
    if (ipart >= s.spec_first[k] && ipart < s.spec_first[k] + s.spec_count[k]) sp = k;
  FSum acc;
  const float inv2s2 = (float)s.spr_inv2s2[level][sp];
  const bool sho = s.sho_omega[sp] > 0;
  const float sa = s.sho_a[level][sp], sb = s.sho_b[level][sp];
  const bool prim = s.prim_a[sp] != 0 || s.prim_b[sp] != 0;
  const float pa = (float)s.prim_a[sp], pb = (float)s.prim_b[sp];
  const float ktau = (float)(s.tau * nStride);
  int tb[kMaxTables], tjb[kMaxTables], tn[kMaxTables], nt = 0;
  if (s.coulomb) {
    for (int ti = 0; ti < s.ntab; ++ti) {
      const DevTable& t = s.tab[ti];
      if (ipart >= t.ifirst1 && ipart < t.ifirst1 + t.npart1) {
        tb[nt] = ti;
        tjb[nt] = t.ifirst2;
        tn[nt++] = t.npart2;
      } else if (ipart >= t.ifirst2 && ipart < t.ifirst2 + t.npart2) {
        tb[nt] = ti;
        tjb[nt] = t.ifirst1;
        tn[nt++] = t.npart1;
      }
    }
  }
  int total = nlinks;
  for (int q = 0; q < nt; ++q) total += tn[q] * nlinks;
  for (int item = tid; item < total; item += nthreads) {
    if (item < nlinks) {
      const int k = item + 1;
      const int t1 = k * nStride, t0 = t1 - nStride;
      const double n1x = m.mx[t1], n1y = m.my[t1], n1z = m.mz[t1];
      const double n0x = m.mx[t0], n0y = m.my[t0], n0z = m.mz[t0];
      const double o1x = m.s1x[t1 * np + ipart], o1y = m.s1y[t1 * np + ipart], o1z = m.s1z[t1 * np + ipart];
      const double o0x = m.s1x[t0 * np + ipart], o0y = m.s1y[t0 * np + ipart], o0z = m.s1z[t0 * np + ipart];
      if (s.spring) {
        float fx, fy, fz, gx, gy, gz;
        pbc_f(s, n1x - n0x, n1y - n0y, n1z - n0z, fx, fy, fz);
        pbc_f(s, o1x - o0x, o1y - o0y, o1z - o0z, gx, gy, gz);
        acc.add(inv2s2 * ((fx * fx + fy * fy + fz * fz) - (gx * gx + gy * gy + gz * gz)));
      }
      if (sho) {
        const float a0x = (float)n0x, a0y = (float)n0y, a0z = (float)n0z;
        const float a1x = (float)n1x, a1y = (float)n1y, a1z = (float)n1z;
        const float b0x = (float)o0x, b0y = (float)o0y, b0z = (float)o0z;
        const float b1x = (float)o1x, b1y = (float)o1y, b1z = (float)o1z;
        const float dnx = (float)(n1x - n0x), dny = (float)(n1y - n0y), dnz = (float)(n1z - n0z);
        const float dox = (float)(o1x - o0x), doy = (float)(o1y - o0y), doz = (float)(o1z - o0z);
        const float dd = (dnx * dnx + dny * dny + dnz * dnz) - (dox * dox + doy * doy + doz * doz);
        const float rr = (a0x * a1x + a0y * a1y + a0z * a1z) - (b0x * b1x + b0y * b1y + b0z * b1z);
        acc.add(sa * dd + sb * rr);
      }
      if (prim && k < nlinks) {
        float xn, yn, zn, xo, yo, zo;
        pbc_f(s, n1x, n1y, n1z, xn, yn, zn);
        pbc_f(s, o1x, o1y, o1z, xo, yo, zo);
        const float r2n = xn * xn + yn * yn + zn * zn, r2o = xo * xo + yo * yo + zo * zo;
        acc.add((pa * (r2n - r2o) + pb * (r2n * r2n - r2o * r2o)) * ktau);
      }
      continue;
    }
    int it = item - nlinks, q = 0;
    while (it >= tn[q] * nlinks) {
      it -= tn[q] * nlinks;
      ++q;
    }
    const DevTable& t = s.tab[tb[q]];
    const int jj = it / nlinks;
    const int j = tjb[q] + jj;
    if (j == ipart) continue;
    const int k = it - jj * nlinks + 1;
    const int t1 = k * nStride, t0 = t1 - nStride;
    const double pjx1 = m.s1x[t1 * np + j], pjy1 = m.s1y[t1 * np + j], pjz1 = m.s1z[t1 * np + j];
    const double pjx0 = m.s1x[t0 * np + j], pjy0 = m.s1y[t0 * np + j], pjz0 = m.s1z[t0 * np + j];
    const bool offdiag = level < 3 && t.norder > 0;
    float actf[2];
#pragma unroll
    for (int pass = 0; pass < 2; ++pass) {
      double ax, ay, az, bx, by, bz;
      if (pass == 0) {
        ax = m.mx[t1]; ay = m.my[t1]; az = m.mz[t1];
        bx = m.mx[t0]; by = m.my[t0]; bz = m.mz[t0];
      } else {
        ax = m.s1x[t1 * np + ipart]; ay = m.s1y[t1 * np + ipart]; az = m.s1z[t1 * np + ipart];
        bx = m.s1x[t0 * np + ipart]; by = m.s1y[t0 * np + ipart]; bz = m.s1z[t0 * np + ipart];
      }
      float fx, fy, fz, gx, gy, gz;
      pbc_f(s, ax - pjx1, ay - pjy1, az - pjz1, fx, fy, fz);
      pbc_f(s, bx - pjx0, by - pjy0, bz - pjz0, gx, gy, gz);
      const float r = sqrtf(fx * fx + fy * fy + fz * fz);
      const float rp = sqrtf(gx * gx + gy * gy + gz * gz);
      const float qq = 0.5f * (r + rp);
      const float sx = fx - gx, sy = fy - gy, sz = fz - gz;
      const float s2 = offdiag ? __fdividef(sx * sx + sy * sy + sz * sz, qq * qq) : 0.f;
      actf[pass] = tab_uk0_f(t, qq, s2, offdiag ? t.norder : 0) * (float)nStride;
    }
    acc.add(actf[0] - actf[1]);
  }
  return acc.value();
}

// e^{ik.r} factor tables of one bead, column `col` of X [nx][w], Y [ny][w] and
// Z [nz][w] (Y and Z rows offset by ikmax): EwaldSum's recurrence over
// multiples of the first wave vector (src/util/EwaldSum.cc:110-150), in
// individually rounded operations, so every kernel that builds a bead's tables
// gets the same bits.
static __device__ __forceinline__ double2 cmul_rn(double2 a, double2 b) {
  return make_double2(__dsub_rn(__dmul_rn(a.x, b.x), __dmul_rn(a.y, b.y)),
                      __dadd_rn(__dmul_rn(a.x, b.y), __dmul_rn(a.y, b.x)));
}

static __device__ void ewald_bead_tables(const DevSys& s, double2* X, double2* Y, double2* Z,
                                         int w, int col, double x, double y, double z) {
  const int kx0 = s.ikmax[0], ky0 = s.ikmax[1], kz0 = s.ikmax[2];
  X[col] = make_double2(1.0, 0.0);
  Y[ky0 * w + col] = make_double2(1.0, 0.0);
  Z[kz0 * w + col] = make_double2(1.0, 0.0);
  double sn, cs;
  if (kx0 > 0) {
    sincos(__dmul_rn(s.deltak[0], x), &sn, &cs);
    X[w + col] = make_double2(cs, sn);
  }
  if (ky0 > 0) {
    sincos(__dmul_rn(s.deltak[1], y), &sn, &cs);
    Y[(ky0 + 1) * w + col] = make_double2(cs, sn);
    Y[(ky0 - 1) * w + col] = make_double2(cs, -sn);
  }
  if (kz0 > 0) {
    sincos(__dmul_rn(s.deltak[2], z), &sn, &cs);
    Z[(kz0 + 1) * w + col] = make_double2(cs, sn);
    Z[(kz0 - 1) * w + col] = make_double2(cs, -sn);
  }
  const double2 x1 = X[w + col];
  for (int k = 2; k <= kx0; ++k) X[k * w + col] = cmul_rn(X[(k - 1) * w + col], x1);
  const double2 yp = Y[(ky0 + 1) * w + col], ym = Y[(ky0 - 1) * w + col];
  for (int k = 2; k <= ky0; ++k) {
    Y[(ky0 + k) * w + col] = cmul_rn(Y[(ky0 + k - 1) * w + col], yp);
    Y[(ky0 - k) * w + col] = cmul_rn(Y[(ky0 - k + 1) * w + col], ym);
  }
  const double2 zp = Z[(kz0 + 1) * w + col], zm = Z[(kz0 - 1) * w + col];
  for (int k = 2; k <= kz0; ++k) {
    Z[(kz0 + k) * w + col] = cmul_rn(Z[(kz0 + k - 1) * w + col], zp);
    Z[(kz0 - k) * w + col] = cmul_rn(Z[(kz0 - k + 1) * w + col], zm);
  }
}

// q e^{ik.r} of table column col for k-vector k, on the fixed-point grid of the
// structure-factor cache (rounded to the nearest multiple of 1/ek_scale).
static __device__ __forceinline__ void ewald_term_fixed(const DevSys& s, const double2* X,
                                                        const double2* Y, const double2* Z,
                                                        int w, int col, int kx, int ky, int kz,
                                                        double q, long long& re, long long& im) {
  const double2 a = X[kx * w + col];
  const double2 t = make_double2(__dmul_rn(q, a.x), __dmul_rn(q, a.y));
  const double2 v = cmul_rn(cmul_rn(t, Y[ky * w + col]), Z[kz * w + col]);
  re = __double2ll_rn(__dmul_rn(v.x, s.ek_scale));
  im = __double2ll_rn(__dmul_rn(v.y, s.ek_scale));
}

// EwaldSum::evalLongRange (src/util/EwaldSum.cc:103-181) for the old and the
// new configuration of one slice (the new one has particle ipart at the moving
// bead), as CoulombAction::getActionDifference uses them at level 0
// (src/action/CoulombAction.cc:107-119).  Returns both evalLongRange values.
static __device__ void ewald_slice_sums(const DevSys& s, const Smem& m, int ipart, int t, double& eold,
                                 double& enew) {
  const int np = s.npart;
  const int kx0 = s.ikmax[0], ky0 = s.ikmax[1], kz0 = s.ikmax[2];
  const int nx = kx0 + 1, ny = 2 * ky0 + 1;
  const int w = m.ewt_cols;            // >= np + 1: column np = moved bead
  double2* X = (double2*)m.ewt;        // [nx][w]
  double2* Y = X + nx * w;             // [ny][w]
  double2* Z = Y + ny * w;             // [nz][w]
  __syncthreads();
  for (int p = threadIdx.x; p < w; p += blockDim.x) {
    if (p < np)
      ewald_bead_tables(s, X, Y, Z, w, p, m.s1x[t * np + p], m.s1y[t * np + p], m.s1z[t * np + p]);
    else
      ewald_bead_tables(s, X, Y, Z, w, p, m.mx[t], m.my[t], m.mz[t]);
  }
  __syncthreads();
  double so = 0.0, sn_ = 0.0;
  for (int k = threadIdx.x; k < s.totk; k += blockDim.x) {
    const int kx = __ldg(s.kvec + 3 * k), ky = __ldg(s.kvec + 3 * k + 1) + ky0,
              kz = __ldg(s.kvec + 3 * k + 2) + kz0;
    double cor = 0, coi = 0, cnr = 0, cni = 0;
    for (int j = 0; j < np; ++j) {
      const int jj = (j == ipart) ? np : j;
      const double qj = m.qpart[j];
      double2 a = X[kx * w + j];
      double tr = qj * a.x, ti = qj * a.y;
      double2 b = Y[ky * w + j];
      double ur = tr * b.x - ti * b.y, ui = tr * b.y + ti * b.x;
      b = Z[kz * w + j];
      const double vr = ur * b.x - ui * b.y, vi = ur * b.y + ui * b.x;
      cor += vr;
      coi += vi;
      if (jj == j) {
        cnr += vr;
        cni += vi;
      } else {
        a = X[kx * w + jj];
        tr = qj * a.x;
        ti = qj * a.y;
        b = Y[ky * w + jj];
        ur = tr * b.x - ti * b.y;
        ui = tr * b.y + ti * b.x;
        b = Z[kz * w + jj];
        cnr += ur * b.x - ui * b.y;
        cni += ur * b.y + ui * b.x;
      }
    }
    const double vk = __ldg(s.vk + k);
    so += 2 * vk * (cor * cor + coi * coi);
    sn_ += 2 * vk * (cnr * cnr + cni * cni);
  }
  const double old_sum = block_sum(so, m.red);
  const double new_sum = block_sum(sn_, m.red);
  eold = old_sum * s.one_over_2v + s.self_energy;
  enew = new_sum * s.one_over_2v + s.self_energy;
}

// (new - old) * tau / epsilon of one slice, the level-0 Ewald term.
static __device__ double ewald_slice_diff(const DevSys& s, const Smem& m, int ipart, int t) {
  double eold, enew;
  ewald_slice_sums(s, m, ipart, t, eold, enew);
  return -(eold * s.tau / s.epsilon) + enew * s.tau / s.epsilon;
}

// evalLongRange of section slice t as staged in shared memory.
static __device__ double ewald_slice_energy(const DevSys& s, const Smem& m, int t) {
  double eold, enew;
  ewald_slice_sums(s, m, -1, t, eold, enew);
  return eold;
}

}  // namespace pimc
