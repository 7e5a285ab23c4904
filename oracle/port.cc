// CPU restatement of pi-qmc's bisection / fixed-node hot path, in plain C++.
// TEST INFRASTRUCTURE: the checker for the CUDA engine on machines where the
// reference tree (and so oracle/_ref) is absent.  Only tests/, the smoke entry
// point and bench.py's CPU-baseline leg load it.  Each routine cites the
// reference code it restates; the arithmetic follows the reference's order of
// operations so results agree to rounding.  Its agreement with the reference
// itself is pinned by tests against oracle/_ref and tests/golden.
//
// Scope: identity permutations (distinguishable particles / fixed node),
// one moving particle, no delayed rejection, no exchange term in the pair
// action (exLevel < 0), norder terms without the z expansion (hasZ = false).
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <complex>
#include <vector>

#include "../pi-qmc_gb300/csrc/pimc_rng.h"
#include "oracle_api.h"

namespace {

typedef std::complex<double> cplx;

struct V3 {
  double x[3];
};

static inline double dot3(const double* a, const double* b) {
  // blitz::dot on TinyVector<double,3>: (a0 b0 + a1 b1) + a2 b2
  return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}

// SuperCell::pbc (src/util/SuperCell.cc:25-34).
struct Cell {
  double a[3], b[3], rcut2;
  void init(const double* L) {
    for (int d = 0; d < 3; ++d) {
      a[d] = L[d];
      b[d] = 1. / L[d];
    }
    double l2 = a[0] * a[0];
    rcut2 = l2;
    for (int i = 1; i < 3; ++i) {
      l2 = a[i] * a[i];
      rcut2 = (rcut2 > l2) ? l2 : rcut2;
    }
    rcut2 *= 0.25;
  }
  void pbc(double* v) const {
    if (dot3(v, v) > rcut2) {
      for (int d = 0; d < 3; ++d) {
        double i = floor(b[d] * v[d] + 1000.5) - 1000;
        v[d] -= a[d] * i;
      }
    }
  }
};

// PeriodicGaussian (src/util/PeriodicGaussian.cc:7-40).
struct PGauss {
  double alpha, length, nome, prefactor, k;
  int nmax;
  mutable double value, gradient;
  static int numberOfTerms(double alpha, double length) {
    return 1 + int(2.0 * sqrt(alpha * length * length));
  }
  void init(double al, double len) {
    const double PI = 3.141592653589793;
    alpha = al;
    length = len;
    nome = exp(-PI * PI / (alpha * length * length));
    nmax = numberOfTerms(alpha, length);
    prefactor = sqrt(PI / (alpha * length * length));
    k = 2 * PI / length;
  }
  double evaluate(double x) const {
    cplx w = exp(cplx(0, k * x));
    cplx sum0 = 0, sum1 = 0;
    cplx ik = cplx(0, k);
    cplx term = 1.0;
    double nomeN = 1.0;
    for (int n = 1; n < nmax; ++n) {
      term *= nomeN * nomeN * nome * w;
      sum0 += term;
      sum1 += term * ik * double(n);
      nomeN *= nome;
    }
    value = prefactor * (1 + 2 * real(sum0));
    gradient = prefactor * 2 * real(sum1);
    return value;
  }
};

struct PairTab {
  int s1, s2;  // species indices
  int ifirst1, npart1, ifirst2, npart2;
  int ngpts, norder, ndata;
  double rgridinv, logrratioinv;
  std::vector<double> ugrid;  // (ngpts,2,ndata)
  double g(int i, int t, int k) const { return ugrid[(i * 2 + t) * ndata + k]; }
  // PairAction::u00 / uk0 / uk0CalcDerivatives (src/action/PairAction.cc:601-655).
  void locate(double q, int& i, double& x) const {
    q *= rgridinv;
    x = log(q) * logrratioinv;
    i = (int)x;
    if (q < 1) {
      i = 0;
      x = 0;
    } else if (i > ngpts - 2) {
      i = ngpts - 2;
      x = 1;
    } else {
      x -= i;
    }
  }
  double u00(double r) const {
    int i;
    double x;
    locate(r, i, x);
    return (1 - x) * g(i, 0, 0) + x * g(i + 1, 0, 0);
  }
  double uk0(double q, double s2) const {
    int i;
    double x;
    locate(q, i, x);
    double action = 0;
    for (int k = norder; k >= 0; k--) {
      action *= s2;
      action += (1 - x) * g(i, 0, k) + x * g(i + 1, 0, k);
    }
    return action;
  }
  // uk0CalcDerivatives with the q and s^2 derivatives (src/action/PairAction.cc:641-660).
  void uk0dd(double q, double s2, double& u, double& utau, double& uq, double& us2) const {
    q *= rgridinv;
    double x = log(q) * logrratioinv;
    int i = (int)x;
    if (q < 1) {
      i = 0;
      x = 0;
    } else if (i > ngpts - 2) {
      i = ngpts - 2;
      x = 1;
    } else {
      x -= i;
    }
    u = utau = uq = us2 = 0;
    for (int k = norder; k >= 0; k--) {
      u *= s2;
      u += (1 - x) * g(i, 0, k) + x * g(i + 1, 0, k);
      utau *= s2;
      utau += (1 - x) * g(i, 1, k) + x * g(i + 1, 1, k);
      uq *= s2;
      uq += g(i + 1, 0, k) - g(i, 0, k);
    }
    uq *= logrratioinv * rgridinv / q;
    for (int k = norder; k > 0; k--) {
      us2 *= s2;
      us2 += k * ((1 - x) * g(i, 0, k) + x * g(i + 1, 0, k));
    }
  }
  void uk0d(double q, double s2, double& u, double& utau) const {
    int i;
    double x;
    locate(q, i, x);
    u = utau = 0;
    for (int k = norder; k >= 0; k--) {
      u *= s2;
      u += (1 - x) * g(i, 0, k) + x * g(i + 1, 0, k);
      utau *= s2;
      utau += (1 - x) * g(i, 1, k) + x * g(i + 1, 1, k);
    }
  }
};

struct Ewald {
  int totk = 0, ikmax[3] = {0, 0, 0};
  std::vector<int> kvec;
  std::vector<double> vk, q;
  double deltak[3], oneOver2V = 0, selfEnergy = 0;
  // EwaldSum::evalLongRange (src/util/EwaldSum.cc:103-181).
  double evalLongRange(const std::vector<V3>& r) const {
    const int np = (int)r.size();
    const int nx = ikmax[0] + 1, ny = 2 * ikmax[1] + 1, nz = 2 * ikmax[2] + 1;
    std::vector<cplx> ex(nx * np), ey(ny * np), ez(nz * np);
    auto X = [&](int k, int i) -> cplx& { return ex[k * np + i]; };
    auto Y = [&](int k, int i) -> cplx& { return ey[(k + ikmax[1]) * np + i]; };
    auto Z = [&](int k, int i) -> cplx& { return ez[(k + ikmax[2]) * np + i]; };
    const cplx I(0, 1);
    for (int i = 0; i < np; ++i) X(0, i) = Y(0, i) = Z(0, i) = 1.0;
    if (ikmax[0] > 0)
      for (int i = 0; i < np; ++i) X(1, i) = exp(I * deltak[0] * r[i].x[0]);
    if (ikmax[1] > 0)
      for (int i = 0; i < np; ++i) {
        Y(1, i) = exp(I * deltak[1] * r[i].x[1]);
        Y(-1, i) = conj(Y(1, i));
      }
    if (ikmax[2] > 0)
      for (int i = 0; i < np; ++i) {
        Z(1, i) = exp(I * deltak[2] * r[i].x[2]);
        Z(-1, i) = conj(Z(1, i));
      }
    for (int kx = 2; kx <= ikmax[0]; ++kx)
      for (int i = 0; i < np; ++i) X(kx, i) = X(kx - 1, i) * X(1, i);
    for (int ky = 2; ky <= ikmax[1]; ++ky)
      for (int i = 0; i < np; ++i) {
        Y(ky, i) = Y(ky - 1, i) * Y(1, i);
        Y(-ky, i) = Y(-ky + 1, i) * Y(-1, i);
      }
    for (int kz = 2; kz <= ikmax[2]; ++kz)
      for (int i = 0; i < np; ++i) {
        Z(kz, i) = Z(kz - 1, i) * Z(1, i);
        Z(-kz, i) = Z(-kz + 1, i) * Z(-1, i);
      }
    double sum = 0;
    for (int k = 0; k < totk; ++k) {
      cplx csum = 0.;
      const int* kv = &kvec[3 * k];
      for (int j = 0; j < np; ++j) csum += q[j] * X(kv[0], j) * Y(kv[1], j) * Z(kv[2], j);
      sum += 2 * vk[k] * norm(csum);
    }
    return sum * oneOver2V + selfEnergy;
  }
};

// Dense LU with partial pivoting (LAPACK dgetrf semantics: first largest |pivot|,
// row interchanges), determinant from the U diagonal and the pivots, and the
// inverse (dgetri semantics).  a is column-major n x n, overwritten by the inverse.
static int lu_det_inverse(double* a, int n, double* det) {
  std::vector<int> piv(n);
  int info = 0;
  for (int j = 0; j < n; ++j) {
    int p = j;
    double amax = fabs(a[j + j * n]);
    for (int i = j + 1; i < n; ++i)
      if (fabs(a[i + j * n]) > amax) {
        amax = fabs(a[i + j * n]);
        p = i;
      }
    piv[j] = p;
    if (a[p + j * n] != 0.0) {
      if (p != j)
        for (int k = 0; k < n; ++k) {
          double t = a[j + k * n];
          a[j + k * n] = a[p + k * n];
          a[p + k * n] = t;
        }
      const double rinv = 1.0 / a[j + j * n];
      for (int i = j + 1; i < n; ++i) a[i + j * n] *= rinv;
    } else if (info == 0) {
      info = j + 1;
    }
    for (int k = j + 1; k < n; ++k) {
      const double ajk = a[j + k * n];
      if (ajk != 0.0)
        for (int i = j + 1; i < n; ++i) a[i + k * n] -= a[i + j * n] * ajk;
    }
  }
  double d = 1;
  for (int i = 0; i < n; ++i) {
    d *= a[i + i * n];
    d *= (piv[i] == i) ? 1 : -1;
  }
  *det = d;
  if (info != 0) return info;
  // Inverse: solve A X = I column by column with the factors.
  std::vector<double> inv(n * n), col(n);
  for (int c = 0; c < n; ++c) {
    for (int i = 0; i < n; ++i) col[i] = (i == c) ? 1.0 : 0.0;
    for (int j = 0; j < n; ++j)
      if (piv[j] != j) {
        double t = col[j];
        col[j] = col[piv[j]];
        col[piv[j]] = t;
      }
    for (int j = 0; j < n; ++j)
      for (int i = j + 1; i < n; ++i) col[i] -= a[i + j * n] * col[j];
    for (int j = n - 1; j >= 0; --j) {
      col[j] /= a[j + j * n];
      for (int i = 0; i < j; ++i) col[i] -= a[i + j * n] * col[j];
    }
    for (int i = 0; i < n; ++i) inv[i + c * n] = col[i];
  }
  memcpy(a, inv.data(), sizeof(double) * n * n);
  return 0;
}

// Node model for one species: SHONodes (src/fixednode/SHONodes.cc:22-170) or
// FreeParticleNodes without updates/Hungarian/iterations
// (src/fixednode/FreeParticleNodes.cc:23-234).
struct NodeModel {
  int kind = 0;  // 1 SHO, 2 free particle
  int npart = 0, ifirst = 0, nslot = 0;
  double tau, mass, omega, temperature, coshwt, sinhwt, c, scale = 1.0;
  const Cell* cell = 0;
  PGauss pg[3];
  std::vector<double> matrix;  // nslot x (npart*npart) column-major inverses
  int nerror = 0;

  double* mat(int islice) { return &matrix[(size_t)islice * npart * npart]; }

  void build(const std::vector<V3>& r1, const std::vector<V3>& r2, double* m) const {
    for (int j = 0; j < npart; ++j) {
      const double* rj = r1[j + ifirst].x;
      for (int i = 0; i < npart; ++i) {
        const double* ri = r2[i + ifirst].x;
        if (kind == 1) {
          double rj2 = dot3(rj, rj), ri2 = dot3(ri, ri), rirj = dot3(ri, rj);
          m[i + j * npart] = scale * exp(-c * ((ri2 + rj2) * coshwt - 2.0 * rirj));
        } else {
          double delta[3] = {rj[0] - ri[0], rj[1] - ri[1], rj[2] - ri[2]};
          cell->pbc(delta);
          double ear2 = scale;
          for (int d = 0; d < 3; ++d) ear2 *= pg[d].evaluate(delta[d]);
          m[i + j * npart] = ear2;
        }
      }
    }
  }

  // NodeModel::evaluate with the rescaling loop.
  int evaluate(const std::vector<V3>& r1, const std::vector<V3>& r2, int islice,
               bool scaleMagnitude, double* detOut) {
    int err = 0;
    double det = 0;
    int guard = 0;
    do {
      err = 0;
      double* m = mat(islice);
      build(r1, r2, m);
      int info = lu_det_inverse(m, npart, &det);
      if (info != 0) {
        err = 1;
        nerror++;
      }
      if (scaleMagnitude && !err && (fabs(det) < 1e-50 || fabs(det) > 1e50)) {
        if (fabs(det) < 1e-250)
          scale *= 2;
        else
          scale *= pow(fabs(det), -1. / npart);
      }
      if (++guard > 4000) break;  // the reference would loop until exit()
    } while (scaleMagnitude && (err || fabs(det) < 1e-50 || fabs(det) > 1e50));
    *detOut = det;
    return err;
  }

  // evaluateDistance; d1/d2 sized npart (all particles), others set to 200.
  void distance(const std::vector<V3>& r1, const std::vector<V3>& r2, int islice,
                double* d1, double* d2, int ntot) {
    for (int i = 0; i < ntot; ++i) d1[i] = d2[i] = 200;
    const double* m = mat(islice);
    for (int j = 0; j < npart; ++j) {
      double lg[3] = {0, 0, 0};
      const double* rj = r1[j + ifirst].x;
      for (int i = 0; i < npart; ++i) {
        const double* ri = r2[i + ifirst].x;
        double grad[3];
        if (kind == 1) {
          double ri2 = dot3(ri, ri), rj2 = dot3(rj, rj), rirj = dot3(ri, rj);
          double e = exp(-c * ((ri2 + rj2) * coshwt - 2 * rirj));
          for (int d = 0; d < 3; ++d) grad[d] = 2 * c * (ri[d] - coshwt * rj[d]) * e;
        } else {
          double delta[3] = {rj[0] - ri[0], rj[1] - ri[1], rj[2] - ri[2]};
          cell->pbc(delta);
          double value[3];
          for (int d = 0; d < 3; ++d) {
            value[d] = pg[d].evaluate(delta[d]);
            grad[d] = pg[d].gradient / (value[d] + 1e-300);
          }
          for (int d = 0; d < 3; ++d)
            for (int e = 0; e < 3; ++e) grad[e] *= value[d];
        }
        const double w = m[j + i * npart];
        for (int d = 0; d < 3; ++d) lg[d] += w * grad[d] * scale;
      }
      d1[j + ifirst] = sqrt(2 * mass / ((dot3(lg, lg) + 1e-15) * tau));
    }
    for (int i = 0; i < npart; ++i) {
      double lg[3] = {0, 0, 0};
      const double* ri = r2[i + ifirst].x;
      for (int j = 0; j < npart; ++j) {
        const double* rj = r1[j + ifirst].x;
        double grad[3];
        if (kind == 1) {
          double ri2 = dot3(ri, ri), rj2 = dot3(rj, rj), rirj = dot3(ri, rj);
          double e = exp(-c * ((ri2 + rj2) * coshwt - 2 * rirj));
          for (int d = 0; d < 3; ++d) grad[d] = 2 * c * (rj[d] - coshwt * ri[d]) * e;
        } else {
          double delta[3] = {ri[0] - rj[0], ri[1] - rj[1], ri[2] - rj[2]};
          cell->pbc(delta);
          double value[3];
          for (int d = 0; d < 3; ++d) {
            value[d] = pg[d].evaluate(delta[d]);
            grad[d] = pg[d].gradient / (value[d] + 1e-300);
          }
          for (int d = 0; d < 3; ++d)
            for (int e = 0; e < 3; ++e) grad[e] *= value[d];
        }
        const double w = m[j + i * npart];
        for (int d = 0; d < 3; ++d) lg[d] += w * grad[d] * scale;
      }
      d2[i + ifirst] = sqrt(2 * mass / ((dot3(lg, lg) + 1e-15) * tau));
    }
  }
};

struct Sim {
  ora_config cfg;
  int np, ns, nsec, L;
  Cell cell;
  std::vector<int> spec;       // species of particle
  std::vector<double> lambda;  // 0.5/mass
  std::vector<int> spec_first;
  std::vector<V3> path;        // [ns][np]
  std::vector<PairTab> pairs;
  bool has_ewald = false;
  Ewald ewald;
  std::vector<NodeModel> nodes;  // per species
  bool fixed_node = false;
  // mover/spring periodic Gaussians (only built for small boxes).
  std::vector<PGauss> pg_spring, pg_mover;
  std::vector<char> has_pg_spring, has_pg_mover;
  // section state
  std::vector<V3> sec1, sec2, mov1;  // [nsec][np] and [nsec]
  int ifirst1, ifirst2;
  // fixed-node per-species caches
  struct FNState {
    std::vector<double> dm, newdm, dist, newdist;  // dist: [nsec][2][np]
    bool notMySpecies;
  };
  std::vector<FNState> fn;
  uint32_t attempt;
  uint32_t uidx, npair;
  int nerror_init;

  V3& P(int t, int i) { return path[(size_t)t * np + i]; }
  V3& S1(int t, int i) { return sec1[(size_t)t * np + i]; }
  V3& S2(int t, int i) { return sec2[(size_t)t * np + i]; }

  double uniform() { return pimc::stream_uniform(cfg.seed, cfg.replica, attempt, uidx++); }
  void normals(double* out, int n) {
    for (int i = 0; i < n; i += 2) {
      double z0, z1;
      pimc::stream_normal_pair(cfg.seed, cfg.replica, attempt, npair++, &z0, &z1);
      out[i] = z0;
      if (i + 1 < n) out[i + 1] = z1;
    }
  }

  // ---- Actions: Action::getActionDifference for one moving particle ------
  // SpringAction::getActionDifference (src/action/SpringAction.cc:56-98).
  double springDiff(const std::vector<V3>& secB, const std::vector<V3>& mov, int i,
                    int level) {
    const int nStride = 1 << level;
    const int ispec = spec[i];
    double deltaAction = 0;
    for (int islice = nStride; islice < nsec; islice += nStride) {
      const double inv2Sigma2 = 0.25 / (lambda[i] * cfg.tau * nStride);
      double delta[3];
      for (int d = 0; d < 3; ++d) delta[d] = mov[islice].x[d] - mov[islice - nStride].x[d];
      cell.pbc(delta);
      double temp = 1.0;
      for (int d = 0; d < 3; ++d) {
        const int pgi = (level * cfg.nspecies + ispec) * 3 + d;
        if (has_pg_spring[pgi])
          temp *= pg_spring[pgi].evaluate(delta[d]);
        else
          deltaAction += delta[d] * delta[d] * inv2Sigma2;
      }
      temp = 1.0 / temp;
      for (int d = 0; d < 3; ++d)
        delta[d] = secB[(size_t)islice * np + i].x[d] - secB[(size_t)(islice - nStride) * np + i].x[d];
      cell.pbc(delta);
      for (int d = 0; d < 3; ++d) {
        const int pgi = (level * cfg.nspecies + ispec) * 3 + d;
        if (has_pg_spring[pgi])
          temp *= pg_spring[pgi].evaluate(delta[d]);
        else
          deltaAction -= delta[d] * delta[d] * inv2Sigma2;
      }
      deltaAction += log(temp);
    }
    return deltaAction;
  }

  // SHOAction::getActionDifference (src/action/SHOAction.cc:19-65).
  double shoDiff(const std::vector<V3>& secB, const std::vector<V3>& mov, int i, int level,
                 int sp) {
    const int nStride = 1 << level;
    const double omega = cfg.sho_omega[sp], m = cfg.spec_mass[sp];
    double deltaAction = 0;
    double wt = omega * cfg.tau * nStride;
    double sinhwt = sinh(wt), coshwt = cosh(wt);
    double div1 = 1.0 / (2.0 * sinhwt), div2 = 1.0 / (2.0 * cfg.tau * nStride);
    for (int islice = nStride; islice < nsec; islice += nStride) {
      for (int pass = 0; pass < 2; ++pass) {
        const double* r1 = pass == 0 ? mov[islice].x : secB[(size_t)islice * np + i].x;
        const double* r0 =
            pass == 0 ? mov[islice - nStride].x : secB[(size_t)(islice - nStride) * np + i].x;
        double r0r0 = 0, r0r1 = 0, r1r1 = 0, delta2 = 0;
        for (int d = 0; d < 3; ++d) {
          double dd = r1[d] - r0[d];
          r0r0 += r0[d] * r0[d];
          r0r1 += r0[d] * r1[d];
          r1r1 += r1[d] * r1[d];
          delta2 += dd * dd;
        }
        double v = m * omega * ((r1r1 + r0r0) * coshwt - 2.0 * r0r1) * div1 - m * delta2 * div2;
        if (pass == 0)
          deltaAction += v;
        else
          deltaAction -= v;
      }
    }
    return deltaAction;
  }

  // PrimSHOAction::getActionDifference (src/action/PrimSHOAction.cc:21-58).
  double primDiff(const std::vector<V3>& secB, const std::vector<V3>& mov, int i, int level,
                  int sp) {
    const int nStride = 1 << level;
    const double a = cfg.prim_a[sp], b = cfg.prim_b[sp];
    double deltaAction = 0;
    double ktstride = cfg.tau * nStride;
    for (int islice = nStride; islice < nsec - nStride; islice += nStride) {
      double delta[3];
      for (int d = 0; d < 3; ++d) delta[d] = mov[islice].x[d];
      cell.pbc(delta);
      double x2 = 0;
      for (int d = 0; d < 3; ++d) x2 += delta[d] * delta[d];
      deltaAction += (a * x2 + b * x2 * x2) * ktstride;
      for (int d = 0; d < 3; ++d) delta[d] = secB[(size_t)islice * np + i].x[d];
      cell.pbc(delta);
      x2 = 0;
      for (int d = 0; d < 3; ++d) x2 += delta[d] * delta[d];
      deltaAction -= (a * x2 + b * x2 * x2) * ktstride;
    }
    return deltaAction;
  }

  // PairAction::getActionDifference (src/action/PairAction.cc:219-360), one mover.
  double pairDiff(const PairTab& pt, const std::vector<V3>& secB, const std::vector<V3>& mov,
                  int i, int level) {
    const int nStride = 1 << level;
    int jbegin, jend;
    if (i >= pt.ifirst1 && i < pt.ifirst1 + pt.npart1) {
      jbegin = pt.ifirst2;
      jend = pt.ifirst2 + pt.npart2;
    } else if (i >= pt.ifirst2 && i < pt.ifirst2 + pt.npart2) {
      jbegin = pt.ifirst1;
      jend = pt.ifirst1 + pt.npart1;
    } else {
      return 0;
    }
    double deltaAction = 0;
    for (int j = jbegin; j < jend; ++j) {
      if (j == i) continue;  // the moving particle itself (isMoving && i<=j)
      double prevDelta[3];
      for (int d = 0; d < 3; ++d) prevDelta[d] = secB[i].x[d] - secB[j].x[d];
      cell.pbc(prevDelta);
      double prevMovingDelta[3] = {prevDelta[0], prevDelta[1], prevDelta[2]};
      double prevR = sqrt(dot3(prevDelta, prevDelta));
      double prevMovingR = prevR;
      for (int islice = nStride; islice < nsec; islice += nStride) {
        double action = 0.;
        double delta[3];
        for (int d = 0; d < 3; ++d)
          delta[d] = mov[islice].x[d] - secB[(size_t)islice * np + j].x[d];
        cell.pbc(delta);
        double r = sqrt(dot3(delta, delta));
        double q = 0.5 * (r + prevMovingR);
        if (level < 3 && pt.norder > 0) {
          double sv[3] = {delta[0] - prevMovingDelta[0], delta[1] - prevMovingDelta[1],
                          delta[2] - prevMovingDelta[2]};
          double s2 = dot3(sv, sv) / (q * q);
          action += pt.uk0(q, s2) * nStride;
        } else {
          action += pt.u00(q) * nStride;
        }
        deltaAction += action;
        for (int d = 0; d < 3; ++d) prevMovingDelta[d] = delta[d];
        prevMovingR = r;
        action = 0.;
        for (int d = 0; d < 3; ++d)
          delta[d] = secB[(size_t)islice * np + i].x[d] - secB[(size_t)islice * np + j].x[d];
        cell.pbc(delta);
        r = sqrt(dot3(delta, delta));
        q = 0.5 * (r + prevR);
        if (level < 3 && pt.norder > 0) {
          double sv[3] = {delta[0] - prevDelta[0], delta[1] - prevDelta[1],
                          delta[2] - prevDelta[2]};
          double s2 = dot3(sv, sv) / (q * q);
          action += pt.uk0(q, s2) * nStride;
        } else {
          action += pt.u00(q) * nStride;
        }
        deltaAction -= action;
        for (int d = 0; d < 3; ++d) prevDelta[d] = delta[d];
        prevR = r;
      }
    }
    return deltaAction;
  }

  // CoulombAction::getActionDifference (src/action/CoulombAction.cc:100-121).
  double coulombDiff(const std::vector<V3>& secB, const std::vector<V3>& mov, int i,
                     int level) {
    double u = 0;
    for (size_t k = 0; k < pairs.size(); ++k) u += pairDiff(pairs[k], secB, mov, i, level);
    if (has_ewald && level == 0) {
      std::vector<V3> rew(np);
      for (int islice = 1; islice < nsec - 1; ++islice) {
        for (int p = 0; p < np; ++p) rew[p] = secB[(size_t)islice * np + p];
        u -= ewald.evalLongRange(rew) * cfg.tau / cfg.epsilon;
        rew[i] = mov[islice];
        u += ewald.evalLongRange(rew) * cfg.tau / cfg.epsilon;
      }
    }
    return u;
  }

  // CompositeAction::getActionDifference (src/action/CompositeAction.cc:30-37), in
  // the order the actions are added: spring, (SHO, PrimSHO) per species, Coulomb.
  double actionDiff(const std::vector<V3>& secB, const std::vector<V3>& mov, int i,
                    int level) {
    double diff = 0;
    if (cfg.spring) diff += springDiff(secB, mov, i, level);
    for (int sp = 0; sp < cfg.nspecies; ++sp) {
      const bool mine = spec[i] == sp;
      if (cfg.sho_omega[sp] > 0) diff += mine ? shoDiff(secB, mov, i, level, sp) : 0.0;
      if (cfg.prim_a[sp] != 0 || cfg.prim_b[sp] != 0)
        diff += mine ? primDiff(secB, mov, i, level, sp) : 0.0;
    }
    if (cfg.coulomb) diff += coulombDiff(secB, mov, i, level);
    return diff;
  }

  // ---- Movers ----------------------------------------------------------
  // FreeMover::makeMove (src/advancer/mover/FreeMover.cc:59-124), at the
  // sampler's current factor; forwardProb as getForwardProb() returns it.
  double forwardProb = 0;
  double freeMove(int i, int level, double factor) {
    const int nStride = 1 << level;
    const int ispec = spec[i];
    double toldOverTnew = 0;
    forwardProb = 0;
    for (int islice = nStride; islice < nsec - nStride; islice += 2 * nStride) {
      double g[3];
      normals(g, 3);
      double sigma = factor * sqrt(lambda[i] * cfg.tau * nStride);
      double inv2Sigma2 = 0.5 / (sigma * sigma);
      double mid[3];
      for (int d = 0; d < 3; ++d) mid[d] = mov1[islice + nStride].x[d] - mov1[islice - nStride].x[d];
      cell.pbc(mid);
      for (int d = 0; d < 3; ++d) mid[d] *= 0.5;
      for (int d = 0; d < 3; ++d) mid[d] += mov1[islice - nStride].x[d];
      cell.pbc(mid);
      double delta[3];
      for (int d = 0; d < 3; ++d) delta[d] = g[d] * sigma;
      cell.pbc(delta);
      for (int d = 0; d < 3; ++d) mov1[islice].x[d] = mid[d] + delta[d];
      cell.pbc(mov1[islice].x);
      double temp = 1.0;
      for (int d = 0; d < 3; ++d) {
        const int pgi = (level * cfg.nspecies + ispec) * 3 + d;
        if (has_pg_mover[pgi]) {
          temp *= pg_mover[pgi].evaluate(delta[d]);
        } else {
          double tmp = delta[d] * delta[d] * inv2Sigma2;
          forwardProb += tmp;
          toldOverTnew += tmp;
        }
      }
      temp = 1.0 / temp;
      forwardProb += log(temp);
      for (int d = 0; d < 3; ++d)
        mid[d] = S1(islice + nStride, i).x[d] - S1(islice - nStride, i).x[d];
      cell.pbc(mid);
      for (int d = 0; d < 3; ++d) mid[d] *= 0.5;
      for (int d = 0; d < 3; ++d) mid[d] += S1(islice - nStride, i).x[d];
      cell.pbc(mid);
      for (int d = 0; d < 3; ++d) delta[d] = S1(islice, i).x[d] - mid[d];
      cell.pbc(delta);
      for (int d = 0; d < 3; ++d) {
        const int pgi = (level * cfg.nspecies + ispec) * 3 + d;
        if (has_pg_mover[pgi])
          temp *= pg_mover[pgi].evaluate(delta[d]);
        else
          toldOverTnew -= delta[d] * delta[d] * inv2Sigma2;
      }
      toldOverTnew += log(temp);
    }
    return toldOverTnew;
  }

  // FreeMover::makeDelayedMove (src/advancer/mover/FreeMover.cc:127-185): the
  // forward probability C->B of the rejected beads `rej` about the midpoints of
  // the current moving beads (C), and the reverse B->C; returns ln(T_old/T_new)
  // and leaves forwardProb.
  double freeDelayedMove(int i, int level, double factor, const std::vector<V3>& rej) {
    const int nStride = 1 << level;
    const int ispec = spec[i];
    double toldOverTnew = 0;
    forwardProb = 0;
    for (int islice = nStride; islice < nsec - nStride; islice += 2 * nStride) {
      double sigma = factor * sqrt(lambda[i] * cfg.tau * nStride);
      double inv2Sigma2 = 0.5 / (sigma * sigma);
      double temp = 1.0;
      double mid[3], delta[3];
      for (int d = 0; d < 3; ++d) mid[d] = mov1[islice + nStride].x[d] - mov1[islice - nStride].x[d];
      cell.pbc(mid);
      for (int d = 0; d < 3; ++d) mid[d] *= 0.5;
      for (int d = 0; d < 3; ++d) mid[d] += mov1[islice - nStride].x[d];
      cell.pbc(mid);
      for (int d = 0; d < 3; ++d) delta[d] = rej[islice].x[d] - mid[d];
      cell.pbc(delta);
      for (int d = 0; d < 3; ++d) {
        const int pgi = (level * cfg.nspecies + ispec) * 3 + d;
        if (has_pg_mover[pgi]) {
          temp *= pg_mover[pgi].evaluate(delta[d]);
        } else {
          double tmp = delta[d] * delta[d] * inv2Sigma2;
          forwardProb -= tmp;
          toldOverTnew += tmp;
        }
      }
      forwardProb += log(temp);
      temp = 1.0 / temp;
      for (int d = 0; d < 3; ++d) mid[d] = rej[islice + nStride].x[d] - rej[islice - nStride].x[d];
      cell.pbc(mid);
      for (int d = 0; d < 3; ++d) mid[d] *= 0.5;
      for (int d = 0; d < 3; ++d) mid[d] += rej[islice - nStride].x[d];
      cell.pbc(mid);
      for (int d = 0; d < 3; ++d) delta[d] = mov1[islice].x[d] - mid[d];
      cell.pbc(delta);
      for (int d = 0; d < 3; ++d) {
        const int pgi = (level * cfg.nspecies + ispec) * 3 + d;
        if (has_pg_mover[pgi])
          temp *= pg_mover[pgi].evaluate(delta[d]);
        else
          toldOverTnew -= delta[d] * delta[d] * inv2Sigma2;
      }
      toldOverTnew += log(temp);
    }
    return toldOverTnew;
  }

  // FreeMoverPBC::makeMove (src/advancer/mover/FreeMoverPBC.cc:59-152).
  double freeMovePBC(int i, int level, double factor) {
    const int nStride = 1 << level;
    const int ispec = spec[i];
    double toldOverTnew = 0.;
    auto pgp = [&](int lev, int d) -> const PGauss* {
      const int k = (lev * cfg.nspecies + ispec) * 3 + d;
      return has_pg_mover[k] ? &pg_mover[k] : (const PGauss*)0;
    };
    for (int islice = nStride; islice < nsec - nStride; islice += 2 * nStride) {
      double g[3];
      normals(g, 3);
      double sigma = factor * sqrt(lambda[i] * cfg.tau * nStride);
      double inv2Sigma2 = 0.5 / (sigma * sigma);
      double mid[3], mid2[3];
      for (int d = 0; d < 3; ++d) mid[d] = mov1[islice + nStride].x[d] - mov1[islice - nStride].x[d];
      cell.pbc(mid);
      for (int d = 0; d < 3; ++d) mid[d] *= 0.5;
      for (int d = 0; d < 3; ++d) mid2[d] = mid[d] + 0.5 * cell.a[d];
      cell.pbc(mid2);
      for (int d = 0; d < 3; ++d) {
        double w1, w2;
        if (const PGauss* p = pgp(level, d)) {
          p->evaluate(mid[d]);
          w1 = p->value;
          p->evaluate(mid2[d]);
          w2 = p->value;
        } else {
          w1 = exp(-inv2Sigma2 * mid[d] * mid[d]);
          w2 = exp(-inv2Sigma2 * mid2[d] * mid2[d]);
        }
        if (uniform() > w1 / (w1 + w2)) mid[d] = mid2[d];
      }
      for (int d = 0; d < 3; ++d) mid[d] += mov1[islice - nStride].x[d];
      for (int d = 0; d < 3; ++d) mov1[islice].x[d] = mid[d] + g[d] * sigma;
      cell.pbc(mov1[islice].x);
      double dpn[3], dnn[3], dn[3], dpo[3], dno[3], dOld[3];
      for (int d = 0; d < 3; ++d) {
        dpn[d] = mov1[islice].x[d] - mov1[islice - nStride].x[d];
        dnn[d] = mov1[islice].x[d] - mov1[islice + nStride].x[d];
        dn[d] = mov1[islice + nStride].x[d] - mov1[islice - nStride].x[d];
        dpo[d] = S1(islice, i).x[d] - S1(islice - nStride, i).x[d];
        dno[d] = S1(islice, i).x[d] - S1(islice + nStride, i).x[d];
        dOld[d] = S1(islice + nStride, i).x[d] - S1(islice - nStride, i).x[d];
      }
      cell.pbc(dpn);
      cell.pbc(dnn);
      cell.pbc(dn);
      cell.pbc(dpo);
      cell.pbc(dno);
      cell.pbc(dOld);
      double temp = 1.;
      for (int d = 0; d < 3; ++d) {
        if (const PGauss* p = pgp(level + 1, d)) {
          temp *= p->evaluate(dpo[d]);
          temp *= p->evaluate(dno[d]);
          temp /= p->evaluate(dpn[d]);
          temp /= p->evaluate(dnn[d]);
        } else {
          toldOverTnew -= dpo[d] * dpo[d] * inv2Sigma2 * 0.5;
          toldOverTnew -= dno[d] * dno[d] * inv2Sigma2 * 0.5;
          toldOverTnew += dpn[d] * dpn[d] * inv2Sigma2 * 0.5;
          toldOverTnew += dnn[d] * dnn[d] * inv2Sigma2 * 0.5;
        }
        if (const PGauss* p = pgp(level + 2, d)) {
          temp /= p->evaluate(dOld[d]);
          temp *= p->evaluate(dn[d]);
        } else {
          toldOverTnew += dOld[d] * dOld[d] * inv2Sigma2 * 0.25;
          toldOverTnew -= dn[d] * dn[d] * inv2Sigma2 * 0.25;
        }
      }
      toldOverTnew += log(temp);
    }
    return toldOverTnew;
  }

  // ---- fixed node -------------------------------------------------------
  void gatherSlice(int islice, bool withMoving, int ipart, std::vector<V3>& r1,
                   std::vector<V3>& r2) {
    for (int p = 0; p < np; ++p) {
      r1[p] = S1(islice, p);
      r2[p] = S2(islice, p);
    }
    if (withMoving) r1[ipart] = mov1[islice];
  }

  // FixedNodeAction::initialize (src/fixednode/FixedNodeAction.cc:331-357).
  void fnInitialize(int sp) {
    NodeModel& nm = nodes[sp];
    FNState& st = fn[sp];
    std::vector<V3> r1(np), r2(np);
    for (int islice = 0; islice < nsec; ++islice) {
      gatherSlice(islice, false, 0, r1, r2);
      double det;
      int err = nm.evaluate(r1, r2, islice, true, &det);
      st.dm[islice] = det;
      if (err || st.dm[islice] * st.dm[0] <= 1e-200) nerror_init++;
      nm.distance(r1, r2, islice, &st.dist[(islice * 2 + 0) * np], &st.dist[(islice * 2 + 1) * np],
                  np);
    }
    st.newdm[0] = st.dm[0];
    for (int k = 0; k < 2 * np; ++k) st.newdist[k] = st.dist[k];
  }

  // FixedNodeAction::getActionDifference (src/fixednode/FixedNodeAction.cc:39-131).
  double fnDiff(int sp, int ipart, int level) {
    NodeModel& nm = nodes[sp];
    FNState& st = fn[sp];
    if (!(ipart >= nm.ifirst && ipart < nm.ifirst + nm.npart)) {
      st.notMySpecies = true;
      return 0;
    }
    st.notMySpecies = false;
    double deltaAction = 0;
    const int nStride = 1 << (level + 1);
    std::vector<V3> r1(np), r2(np);
    for (int islice = nStride / 2; islice < nsec; islice += nStride) {
      gatherSlice(islice, true, ipart, r1, r2);
      double det;
      int err = nm.evaluate(r1, r2, islice, false, &det);
      if (err) return deltaAction = 2e100;
      st.newdm[islice] = det;
      if (st.newdm[islice] * st.dm[0] <= 1e-200) return deltaAction = 2e100;
    }
    if (level == 0) {
      for (int islice = 1; islice < nsec; ++islice) {
        gatherSlice(islice, true, ipart, r1, r2);
        nm.distance(r1, r2, islice, &st.newdist[(islice * 2 + 0) * np],
                    &st.newdist[(islice * 2 + 1) * np], np);
        for (int p = 0; p < np; ++p) {
          const double* D = &st.dist[0];
          const double* N = &st.newdist[0];
          auto at = [&](const double* A, int s, int w) { return A[(s * 2 + w) * np + p]; };
          deltaAction += log((1 - exp(-at(D, islice, 0) * at(D, islice - 1, 0))) /
                             (1 - exp(-at(N, islice, 0) * at(N, islice - 1, 0))));
          deltaAction += log((1 - exp(-at(D, islice, 1) * at(D, islice - 1, 1))) /
                             (1 - exp(-at(N, islice, 1) * at(N, islice - 1, 1))));
        }
      }
    }
    return deltaAction;
  }

  void fnAccept(int sp) {
    FNState& st = fn[sp];
    if (st.notMySpecies) return;
    st.dm = st.newdm;
    st.dist = st.newdist;
  }

  // ---- section bookkeeping (SerialPaths::getBeads/putBeads, identity perm) --
  void getBeads(int ifirst, std::vector<V3>& out) {
    for (int k = 0; k < nsec; ++k) {
      int islice = k + ifirst;
      int t = islice < 0 ? islice + ns : (islice < ns ? islice : islice - ns);
      for (int p = 0; p < np; ++p) out[(size_t)k * np + p] = P(t, p);
    }
  }
  void putBeads(int ifirst, const std::vector<V3>& in) {
    for (int k = 0; k < nsec; ++k) {
      int islice = k + ifirst;
      if (islice < 0) continue;
      int t = islice < ns ? islice : islice % ns;
      for (int p = 0; p < np; ++p) P(t, p) = in[(size_t)k * np + p];
    }
  }

  // MultiLevelSampler::tryMove / DoubleMLSampler::tryMove
  // (src/advancer/MultiLevelSampler.cc:100-177, src/advancer/DoubleMLSampler.cc:123-245).
  // With delayedRejection, level L - 1's rejected first proposal B gets a
  // second proposal C (MultiLevelSampler.cc:114-148, DoubleMLSampler.cc:148-204);
  // the records then hold C's values, as pi-qmc's last calls leave them.
  bool tryMove(int ipart, ora_record* rec) {
    const double defaultFactor = cfg.sigma_factor != 0 ? cfg.sigma_factor : 1.0;
    const double newFactor = cfg.dr_sigma_factor != 0 ? cfg.dr_sigma_factor : 0.75;
    double oldDeltaAction = 0;
    auto propose = [&](int ilevel, double factor, double& lnT, double& dS) {
      lnT = cfg.mover == 1 ? freeMovePBC(ipart, ilevel, factor)
                           : freeMove(ipart, ilevel, factor);
      dS = actionDiff(sec1, mov1, ipart, ilevel);
      double dnode = 0;
      if (fixed_node)
        for (int sp = 0; sp < cfg.nspecies; ++sp)
          if (nodes[sp].kind) dnode += fnDiff(sp, ipart, ilevel);
      if (rec) {
        rec->lnt[ilevel] = lnT;
        rec->ds[ilevel] = dS;
        rec->ds_node[ilevel] = dnode;
      }
      if (fixed_node) dS += dnode;
    };
    for (int ilevel = L; ilevel >= 0; --ilevel) {
      double lnTranProb, deltaAction;
      propose(ilevel, defaultFactor, lnTranProb, deltaAction);
      const double transA2B = forwardProb;
      double piRatioBoA = -deltaAction + oldDeltaAction;
      double acceptProb = exp(lnTranProb + piRatioBoA);
      if (cfg.delayed_rejection && ilevel == L - 1) {
        if (uniform() > acceptProb) {
          double accRatioA2B = acceptProb;
          std::vector<V3> rej(mov1.begin(), mov1.end());
          propose(ilevel, newFactor, lnTranProb, deltaAction);
          double piRatioCoA = -deltaAction + oldDeltaAction;
          double accRatioA2C = exp(lnTranProb + piRatioCoA);
          lnTranProb = freeDelayedMove(ipart, ilevel, defaultFactor, rej);
          double transC2B = forwardProb;
          double accRatioC2B = exp(lnTranProb - piRatioCoA + piRatioBoA);
          accRatioC2B = (accRatioC2B >= 1) ? 1 : accRatioC2B;
          double accRatioA2B2C =
              accRatioA2C * exp(transC2B + transA2B) * (1 - accRatioC2B) / (1 - accRatioA2B);
          deltaAction = deltaAction - transC2B - transA2B -
                        log((1 - accRatioC2B) / (1 - accRatioA2B));
          if (uniform() > accRatioA2B2C) {
            if (rec) rec->reject_level = ilevel;
            return false;
          }
        }
      } else if (uniform() > acceptProb) {
        if (rec) rec->reject_level = ilevel;
        return false;
      }
      oldDeltaAction = deltaAction;
    }
    if (fixed_node)
      for (int sp = 0; sp < cfg.nspecies; ++sp)
        if (nodes[sp].kind) fnAccept(sp);
    for (int islice = 0; islice < nsec; ++islice) S1(islice, ipart) = mov1[islice];
    if (rec) rec->reject_level = -1;
    return true;
  }

  // One section attempt: SectionChooser::run or DoubleSectionChooser::run
  // (src/advancer/SectionChooser.cc:30-48, src/advancer/DoubleSectionChooser.cc:33-65)
  // around one MultiLevelSampler/DoubleMLSampler::run with SimpleParticleChooser.
  bool attemptMove(uint32_t a, ora_record* rec) {
    attempt = a;
    uidx = 0;
    npair = 0;
    if (rec) {
      memset(rec, 0, sizeof(*rec));
      rec->ifirst2 = -2;
    }
    if (!fixed_node) {
      double x = uniform() * (1 - 1e-8);
      int ilo = -1, ihi = ns - 1;
      ifirst1 = ilo + (int)((ihi + 1 - ilo) * x);
      if (ifirst1 > ihi) ifirst1 = ihi;
      getBeads(ifirst1, sec1);
    } else {
      double x = uniform() * (1 - 1e-8);
      int ilo = -1, ihi = ns / 2 - 1;
      ifirst1 = ilo + (int)((ihi + 1 - ilo) * x);
      if (ifirst1 > ihi) ifirst1 = ihi;
      if (uniform() >= 0.5) ifirst1 = (ifirst1 + ns / 2 + 1) % ns - 1;
      ifirst2 = (ifirst1 + ns / 2 + 1) % ns - 1;
      getBeads(ifirst1, sec1);
      getBeads(ifirst2, sec2);
      for (int sp = 0; sp < cfg.nspecies; ++sp)
        if (nodes[sp].kind) fnInitialize(sp);
    }
    if (rec) {
      rec->ifirst1 = ifirst1;
      if (fixed_node) rec->ifirst2 = ifirst2;
    }
    // SimpleParticleChooser::chooseParticles (src/advancer/SimpleParticleChooser.cc:16-28).
    int ipart;
    do {
      ipart = (int)(np * uniform());
    } while (ipart == np);
    if (rec) rec->ipart = ipart;
    mov1[0] = S1(0, ipart);
    mov1[nsec - 1] = S1(nsec - 1, ipart);
    bool acc = tryMove(ipart, rec);
    if (!fixed_node) {
      putBeads(ifirst1, sec1);
    } else if (ifirst1 < ns / 2 - 1) {
      putBeads(ifirst1, sec1);
      putBeads(ifirst2, sec2);
    } else {
      putBeads(ifirst2, sec2);
      putBeads(ifirst1, sec1);
    }
    return acc;
  }

  // ---- estimators --------------------------------------------------------
  const V3& bead(int i, int t) {  // paths(i, t) with wrap (identity permutation)
    int s = t < 0 ? t + ns : (t >= ns ? t - ns : t);
    return P(s, i);
  }
  // Sum over actions of utau at one link, as CompositeAction::getBeadAction
  // (src/action/CompositeAction.cc:59-69) feeding ThermoEnergyEstimator.
  double beadUtau(int ip, int islice) {
    double utau = 0;
    const int sp = spec[ip];
    if (cfg.spring) {  // SpringAction::getBeadAction (src/action/SpringAction.cc:112-123)
      double delta[3];
      for (int d = 0; d < 3; ++d) delta[d] = bead(ip, islice).x[d] - bead(ip, islice - 1).x[d];
      cell.pbc(delta);
      utau += 3 / (2 * cfg.tau) - dot3(delta, delta) / (4.0 * lambda[ip] * cfg.tau * cfg.tau);
    }
    for (int s2 = 0; s2 < cfg.nspecies; ++s2) {
      if (cfg.sho_omega[s2] > 0) {  // SHOAction::getBeadAction (src/action/SHOAction.cc:71-105)
        double ut = 0;
        if (s2 == sp) {
          const double omega = cfg.sho_omega[s2], m = cfg.spec_mass[s2], tau = cfg.tau;
          double wt = omega * tau, sinhwt = sinh(wt), coshwt = cosh(wt);
          double cschwt = 1.0 / sinhwt, cothwt = coshwt * cschwt, tin = 1.0 / tau;
          const double* r1 = bead(ip, islice).x;
          const double* r0 = bead(ip, islice - 1).x;
          double delta[3];
          for (int d = 0; d < 3; ++d) delta[d] = r1[d] - r0[d];
          cell.pbc(delta);
          double r0r0 = 0, r0r1 = 0, r1r1 = 0, delta2 = 0;
          for (int d = 0; d < 3; ++d) {
            r0r0 += r0[d] * r0[d];
            r0r1 += r0[d] * r1[d];
            r1r1 += r1[d] * r1[d];
            delta2 += delta[d] * delta[d];
          }
          ut = 0.5 * 3 * omega * cothwt +
               0.5 * m * omega * omega *
                   ((r1r1 + r0r0) * (1 - cothwt * cothwt) + 2.0 * r0r1 * coshwt * cschwt * cschwt) +
               0.5 * m * delta2 * tin * tin - 0.5 * 3 * tin;
        }
        utau += ut;
      }
      if (cfg.prim_a[s2] != 0 || cfg.prim_b[s2] != 0) {
        double ut = 0;
        if (s2 == sp) {
          const double* x = bead(ip, islice).x;
          double x2 = 0;
          for (int d = 0; d < 3; ++d) x2 += x[d] * x[d];
          ut = cfg.prim_a[s2] * x2 + cfg.prim_b[s2] * x2 * x2;
        }
        utau += ut;
      }
    }
    if (cfg.coulomb) {  // CoulombAction::getBeadAction (src/action/CoulombAction.cc:154-172)
      double ucoul = 0;
      for (size_t k = 0; k < pairs.size(); ++k) {
        const PairTab& pt = pairs[k];
        double up = 0;
        int jbegin, jend;
        if (ip >= pt.ifirst1 && ip < pt.ifirst1 + pt.npart1) {
          jbegin = pt.ifirst2;
          jend = pt.ifirst2 + pt.npart2;
        } else if (ip >= pt.ifirst2 && ip < pt.ifirst2 + pt.npart2) {
          jbegin = pt.ifirst1;
          jend = pt.ifirst1 + pt.npart1;
        } else {
          ucoul += 0.0;
          continue;
        }
        // PairAction::getBeadAction (src/action/PairAction.cc:509-599).
        for (int j = jbegin; j < jend; ++j) {
          if (ip == j) continue;
          double delta[3], prev[3];
          for (int d = 0; d < 3; ++d) delta[d] = bead(ip, islice).x[d] - bead(j, islice).x[d];
          cell.pbc(delta);
          double r = sqrt(dot3(delta, delta));
          for (int d = 0; d < 3; ++d) prev[d] = bead(ip, islice - 1).x[d] - bead(j, islice - 1).x[d];
          cell.pbc(prev);
          double prevR = sqrt(dot3(prev, prev));
          double q = 0.5 * (r + prevR);
          double sv[3] = {delta[0] - prev[0], delta[1] - prev[1], delta[2] - prev[2]};
          double s2 = dot3(sv, sv) / (q * q);
          double v, vtau;
          pt.uk0d(q, s2, v, vtau);
          up += 0.5 * vtau;
        }
        ucoul += up;
      }
      if (has_ewald && ip == 0) {
        std::vector<V3> rew(np);
        for (int p = 0; p < np; ++p) rew[p] = P(islice, p);
        ucoul += ewald.evalLongRange(rew) / cfg.epsilon;
      }
      utau += ucoul;
    }
    return utau;
  }

  double thermoEnergy() {
    double sum = 0;
    for (int ip = 0; ip < np; ++ip) sum += beadUtau(ip, 0);
    for (int islice = 1; islice < ns; ++islice)
      for (int ip = 0; ip < np; ++ip) sum += beadUtau(ip, islice);
    return sum / ns;
  }

  // The forces fm, fp of getBeadAction summed over the actions: SpringAction
  // (src/action/SpringAction.cc:112-123), SHOAction (SHOAction.cc:71-105),
  // PrimSHOAction (PrimSHOAction.cc:65-81), PairAction (PairAction.cc:509-599);
  // the Ewald long-range term and FixedNodeAction add none.
  void beadForces(int ip, int islice, double* fm, double* fp) {
    for (int d = 0; d < 3; ++d) fm[d] = fp[d] = 0;
    const int sp = spec[ip];
    const double tau = cfg.tau;
    if (cfg.spring) {
      double dm[3], dp[3];
      for (int d = 0; d < 3; ++d) {
        dm[d] = bead(ip, islice).x[d] - bead(ip, islice - 1).x[d];
        dp[d] = bead(ip, islice).x[d] - bead(ip, islice + 1).x[d];
      }
      cell.pbc(dm);
      cell.pbc(dp);
      for (int d = 0; d < 3; ++d) {
        fm[d] -= dm[d] / (2 * lambda[ip] * tau);
        fp[d] -= dp[d] / (2 * lambda[ip] * tau);
      }
    }
    if (cfg.sho_omega[sp] > 0) {
      const double omega = cfg.sho_omega[sp], m = cfg.spec_mass[sp];
      const double wt = omega * tau, sinhwt = sinh(wt), coshwt = cosh(wt);
      const double cschwt = 1.0 / sinhwt, tin = 1.0 / tau;
      const double* r1 = bead(ip, islice).x;
      const double* r0 = bead(ip, islice - 1).x;
      const double* r2 = bead(ip, islice + 1).x;
      double dm[3], dp[3];
      for (int d = 0; d < 3; ++d) {
        dm[d] = r1[d] - r0[d];
        dp[d] = r1[d] - r2[d];
      }
      cell.pbc(dm);
      cell.pbc(dp);
      for (int d = 0; d < 3; ++d) {
        fm[d] -= m * omega * (r1[d] * coshwt - r0[d]) * cschwt - m * dm[d] * tin;
        fp[d] -= m * omega * (r1[d] * coshwt - r2[d]) * cschwt - m * dp[d] * tin;
      }
    }
    if (cfg.prim_a[sp] != 0 || cfg.prim_b[sp] != 0) {
      const double* x = bead(ip, islice).x;
      double x2 = 0;
      for (int d = 0; d < 3; ++d) x2 += x[d] * x[d];
      const double a = cfg.prim_a[sp], b = cfg.prim_b[sp];
      for (int d = 0; d < 3; ++d) {
        fm[d] += -0.5 * (2 * a + 4 * b * x2) * tau * x[d];
        fp[d] += -0.5 * (2 * a + 4 * b * x2) * tau * x[d];
      }
    }
    if (cfg.coulomb) {
      for (size_t k = 0; k < pairs.size(); ++k) {
        const PairTab& pt = pairs[k];
        int jbegin, jend;
        if (ip >= pt.ifirst1 && ip < pt.ifirst1 + pt.npart1) {
          jbegin = pt.ifirst2;
          jend = pt.ifirst2 + pt.npart2;
        } else if (ip >= pt.ifirst2 && ip < pt.ifirst2 + pt.npart2) {
          jbegin = pt.ifirst1;
          jend = pt.ifirst1 + pt.npart1;
        } else {
          continue;
        }
        for (int j = jbegin; j < jend; ++j) {
          if (ip == j) continue;
          double delta[3], prev[3], next[3];
          for (int d = 0; d < 3; ++d) {
            delta[d] = bead(ip, islice).x[d] - bead(j, islice).x[d];
            prev[d] = bead(ip, islice - 1).x[d] - bead(j, islice - 1).x[d];
            next[d] = bead(ip, islice + 1).x[d] - bead(j, islice + 1).x[d];
          }
          cell.pbc(delta);
          cell.pbc(prev);
          cell.pbc(next);
          const double r = sqrt(dot3(delta, delta));
          for (int side = 0; side < 2; ++side) {
            const double* o = side == 0 ? prev : next;
            const double ro = sqrt(dot3(o, o));
            const double q = 0.5 * (r + ro);
            double sv[3] = {delta[0] - o[0], delta[1] - o[1], delta[2] - o[2]};
            const double s2 = dot3(sv, sv) / (q * q);
            double v, vtau, vq, vs2;
            pt.uk0dd(q, s2, v, vtau, vq, vs2);
            double* f = side == 0 ? fm : fp;
            for (int d = 0; d < 3; ++d)
              f[d] -= vq * delta[d] / (2 * r) + vs2 * (2 * sv[d] / (q * q) - s2 * delta[d] / (q * r));
          }
        }
      }
    }
  }

  // VirialEnergyEstimator::handleLink / endCalc (src/estimator/VirialEnergyEstimator.cc:34-79)
  // over SerialPaths::sumOverLinks' order (src/base/SerialPaths.cc:48-66).
  double virialEnergy(int nwindow) {
    std::vector<double> r0(3 * np, 0.0), rav(3 * np, 0.0), fav(3 * np, 0.0);
    double energy = 0;
    const double tau = cfg.tau;
    for (int islice = 0; islice < ns; ++islice) {
      for (int ip = 0; ip < np; ++ip) {
        double* R0 = &r0[3 * ip];
        double* RAV = &rav[3 * ip];
        double* FAV = &fav[3 * ip];
        if (islice % nwindow == 0) {
          energy += (1 / (2 * tau)) * dot3(FAV, R0);
          for (int d = 0; d < 3; ++d) R0[d] = RAV[d] = FAV[d] = 0;
        }
        const int thisWindow = (islice / nwindow < (ns - 1) / nwindow) ? nwindow
                                                                        : (ns - 1) % nwindow + 1;
        double r[3];
        for (int d = 0; d < 3; ++d) r[d] = bead(ip, islice).x[d] - bead(ip, islice - 1).x[d];
        cell.pbc(r);
        for (int d = 0; d < 3; ++d) {
          RAV[d] += r[d];
          R0[d] += (thisWindow - islice % nwindow) * r[d] / thisWindow;
        }
        double fm[3], fp[3];
        beadForces(ip, islice, fm, fp);
        const double utau = beadUtau(ip, islice);
        double f[3];
        for (int d = 0; d < 3; ++d) {
          f[d] = fm[d] + fp[d];
          FAV[d] += f[d];
        }
        energy += utau;
        energy += -(1. - 1. / thisWindow) * (3 / (2 * tau)) - (1 / (2 * tau)) * dot3(f, RAV);
      }
    }
    for (int ip = 0; ip < np; ++ip) energy += (1 / (2 * tau)) * dot3(&fav[3 * ip], &r0[3 * ip]);
    return energy / ns;
  }

  // CoulombEnergyEstimator::handleLink (src/estimator/CoulombEnergyEstimator.cc:30-40).
  double coulombEnergy(double epsilon) {
    double e = 0;
    for (int islice = 0; islice < ns; ++islice)
      for (int ip = 0; ip < np; ++ip) {
        double energy = 0;  // one link's sum, then added (ScalarAccumulator::addToValue)
        for (int j = 0; j < ip; ++j) {
          double d[3];
          for (int a = 0; a < 3; ++a) d[a] = bead(ip, islice).x[a] - bead(j, islice).x[a];
          cell.pbc(d);
          energy += charge(ip) * charge(j) / (epsilon * sqrt(dot3(d, d)));
        }
        e += energy;
      }
    return e / ns;
  }

  // EwaldCoulombEstimator::handleLink, optimized-Ewald branch
  // (src/estimator/EwaldCoulombEstimator.cc:102-140): tabulated short range up to
  // rcut (pi-qmc interpolates with x = r - i dr, not divided by dr), plus the
  // long-range sum of each slice.
  double ewaldCoulombEnergy(double epsilon, double rcut, const Ewald& est,
                            const std::vector<double>& vgrid) {
    const double dr = rcut / 1000, drinv = 1. / dr;
    double e = 0;
    for (int islice = 0; islice < ns; ++islice)
      for (int ip = 0; ip < np; ++ip) {
        double energy = 0.0;
        for (int j = 0; j < ip; ++j) {
          double d[3];
          for (int a = 0; a < 3; ++a) d[a] = bead(ip, islice).x[a] - bead(j, islice).x[a];
          cell.pbc(d);
          const double r = sqrt(dot3(d, d));
          if (r < rcut) {
            const int ig = (int)(r * drinv);
            const double x = r - ig * dr;
            energy += charge(ip) * charge(j) *
                      (1. / (r * epsilon) + (1 - x) * vgrid[ig] + x * vgrid[ig + 1]);
          }
        }
        if (ip == 0) {
          std::vector<V3> rew(np);
          for (int p = 0; p < np; ++p) rew[p] = P(islice, p);
          energy += est.evalLongRange(rew) / epsilon;
        }
        e += energy;
      }
    return e / ns;
  }
  double charge(int ip) const { return cfg.spec_charge[spec[ip]]; }

  // ---------------------------------------------------- rigid displacement
  // SHOAction::getActionDifference(Paths, displacement, ...)
  // (src/action/SHOAction.cc:107-143); the loop stops at the first moving
  // particle outside the species, as the reference's `break` does.
  double shoDisplaceDiff(int sp, const std::vector<int>& idx, const std::vector<V3>& disp,
                         int i1, int i2) {
    const double omega = cfg.sho_omega[sp], m = cfg.spec_mass[sp], tau = cfg.tau;
    const double wt = omega * tau, sinhwt = sinh(wt), coshwt = cosh(wt);
    const double div1 = 1.0 / (2.0 * sinhwt);
    const int f = spec_first[sp], n = cfg.spec_count[sp];
    double da = 0;
    for (size_t k = 0; k < idx.size(); ++k) {
      const int ip = idx[k];
      if (ip < f || ip >= f + n) break;
      for (int t = i1; t <= i2; ++t) {
        double r1[3], r0[3];
        for (int d = 0; d < 3; ++d) {
          r1[d] = bead(ip, t).x[d];
          r0[d] = bead(ip, t - 1).x[d];
        }
        da -= m * omega * ((dot3(r1, r1) + dot3(r0, r0)) * coshwt - 2.0 * dot3(r0, r1)) * div1;
        for (int d = 0; d < 3; ++d) {
          r1[d] += disp[k].x[d];
          r0[d] += disp[k].x[d];
        }
        da += m * omega * ((dot3(r1, r1) + dot3(r0, r0)) * coshwt - 2.0 * dot3(r0, r1)) * div1;
      }
    }
    return da;
  }

  // PairAction::getActionDifference(Paths, displacement, ...)
  // (src/action/PairAction.cc:362-500), without the exchange correction.
  double pairDisplaceDiff(const PairTab& pt, const std::vector<int>& idx,
                          const std::vector<V3>& disp, int i1, int i2) {
    double da = 0;
    const int nmov = (int)idx.size();
    for (int im = 0; im < nmov; ++im) {
      const int i = idx[im];
      int jb, je;
      if (i >= pt.ifirst1 && i < pt.ifirst1 + pt.npart1) {
        jb = pt.ifirst2;
        je = pt.ifirst2 + pt.npart2;
      } else if (i >= pt.ifirst2 && i < pt.ifirst2 + pt.npart2) {
        jb = pt.ifirst1;
        je = pt.ifirst1 + pt.npart1;
      } else {
        continue;
      }
      for (int j = jb; j < je; ++j) {
        bool isMoving = false;
        int jm = 0;
        for (int k = 0; k < nmov; ++k)
          if (j == idx[k]) {
            isMoving = true;
            jm = k;
            break;
          }
        if (isMoving && i <= j) continue;
        double prevDelta[3], pmd[3];
        for (int d = 0; d < 3; ++d) prevDelta[d] = bead(i, i1 - 1).x[d] - bead(j, i1 - 1).x[d];
        cell.pbc(prevDelta);
        for (int d = 0; d < 3; ++d) {
          pmd[d] = prevDelta[d] + disp[im].x[d];
          if (isMoving) pmd[d] -= disp[jm].x[d];
        }
        cell.pbc(pmd);
        double prevR = sqrt(dot3(prevDelta, prevDelta)), prevMovingR = sqrt(dot3(pmd, pmd));
        for (int t = i1; t <= i2; ++t) {
          double delta[3];
          for (int d = 0; d < 3; ++d) {
            delta[d] = bead(i, t).x[d] + disp[im].x[d] - bead(j, t).x[d];
            if (isMoving) delta[d] -= disp[jm].x[d];
          }
          cell.pbc(delta);
          double r = sqrt(dot3(delta, delta));
          double q = 0.5 * (r + prevMovingR);
          double action;
          if (pt.norder > 0) {
            double sv[3] = {delta[0] - pmd[0], delta[1] - pmd[1], delta[2] - pmd[2]};
            action = pt.uk0(q, dot3(sv, sv) / (q * q));
          } else {
            action = pt.u00(q);
          }
          da += action;
          for (int d = 0; d < 3; ++d) pmd[d] = delta[d];
          prevMovingR = r;
          for (int d = 0; d < 3; ++d) delta[d] = bead(i, t).x[d] - bead(j, t).x[d];
          cell.pbc(delta);
          r = sqrt(dot3(delta, delta));
          q = 0.5 * (r + prevR);
          if (pt.norder > 0) {
            double sv[3] = {delta[0] - prevDelta[0], delta[1] - prevDelta[1],
                            delta[2] - prevDelta[2]};
            action = pt.uk0(q, dot3(sv, sv) / (q * q));
          } else {
            action = pt.u00(q);
          }
          da -= action;
          for (int d = 0; d < 3; ++d) prevDelta[d] = delta[d];
          prevR = r;
        }
      }
    }
    return da;
  }

  // CompositeAction::getActionDifference(Paths, displacement, ...) over
  // Spring (0), SHO, PrimSHO (the base class's 0) and Coulomb (pairs, then the
  // Ewald long range of every slice, src/action/CoulombAction.cc:123-146).
  double actionDisplaceDiff(const std::vector<int>& idx, const std::vector<V3>& disp, int i1,
                            int i2) {
    double diff = 0;
    for (int sp = 0; sp < cfg.nspecies; ++sp)
      if (cfg.sho_omega[sp] > 0) diff += shoDisplaceDiff(sp, idx, disp, i1, i2);
    if (cfg.coulomb) {
      double u = 0;
      for (size_t k = 0; k < pairs.size(); ++k) u += pairDisplaceDiff(pairs[k], idx, disp, i1, i2);
      if (has_ewald) {
        std::vector<V3> rew(np);
        for (int t = i1; t <= i2; ++t) {
          for (int p = 0; p < np; ++p) rew[p] = bead(p, t);
          u -= ewald.evalLongRange(rew) * cfg.tau / cfg.epsilon;
          for (size_t k = 0; k < idx.size(); ++k) {
            for (int d = 0; d < 3; ++d) rew[idx[k]].x[d] += disp[k].x[d];
            cell.pbc(rew[idx[k]].x);
          }
          u += ewald.evalLongRange(rew) * cfg.tau / cfg.epsilon;
        }
      }
      diff += u;
    }
    return diff;
  }

  // FixedNodeAction::getActionDifference(Paths, displacement, ...)
  // (src/fixednode/FixedNodeAction.cc:133-248) for one species' node model:
  // new configuration (moving particles shifted on both slices of each pair)
  // then the old one, slice pairs (t, t + M/2) for t in [i1, i2].
  double nodeDisplaceDiff(int sp, const std::vector<int>& idx, const std::vector<V3>& disp,
                          int i1, int i2) {
    NodeModel& nm = nodes[sp];
    const int f = spec_first[sp], n = cfg.spec_count[sp];
    for (size_t i = 0; i < idx.size(); ++i) {
      if (idx[i] >= f && idx[i] < f + n) break;
      if (i == idx.size() - 1) return 0;
    }
    const int half = ns / 2;
    std::vector<double> d1(np), d2(np), p1(np), p2(np);
    std::vector<V3> r1(np), r2(np);
    double da = 0, oldDet = 0;
    for (int t = i1; t <= i2; ++t) {
      for (int i = 0; i < np; ++i) {
        r1[i] = bead(i, t);
        r2[i] = bead(i, t + half);
      }
      for (size_t k = 0; k < idx.size(); ++k) {
        for (int d = 0; d < 3; ++d) {
          r1[idx[k]].x[d] += disp[k].x[d];
          r2[idx[k]].x[d] += disp[k].x[d];
        }
        cell.pbc(r1[idx[k]].x);
        cell.pbc(r2[idx[k]].x);
      }
      double det = 0;
      if (nm.evaluate(r1, r2, 0, false, &det)) return 2e100;
      if (t == i1) oldDet = det;
      if (det * oldDet < 0.0) return 2e100;
      nm.distance(r1, r2, 0, d1.data(), d2.data(), np);
      if (t > i1)
        for (int i = 0; i < np; ++i) da -= log((1 - exp(-d1[i] * p1[i])) * (1 - exp(-d2[i] * p2[i])));
      p1 = d1;
      p2 = d2;
    }
    for (int t = i1; t <= i2; ++t) {
      for (int i = 0; i < np; ++i) {
        r1[i] = bead(i, t);
        r2[i] = bead(i, t + half);
      }
      double det = 0;
      if (nm.evaluate(r1, r2, 0, false, &det)) return 2e100;
      nm.distance(r1, r2, 0, d1.data(), d2.data(), np);
      if (t > i1)
        for (int i = 0; i < np; ++i) da += log((1 - exp(-d1[i] * p1[i])) * (1 - exp(-d2[i] * p2[i])));
      p1 = d1;
      p2 = d2;
    }
    return da;
  }

  // One DisplaceMoveSampler::run with nrepeat 1 (DoubleDisplaceMoveSampler for
  // fixed-node systems): SimpleParticleChooser (species < 0) or
  // SpeciesParticleChooser, UniformMover::makeMove (src/advancer/UniformMover.cc:25-42),
  // tryMove (src/advancer/DisplaceMoveSampler.cc:158-224,
  // DoubleDisplaceMoveSampler.cc:40-128).
  bool displaceMove(uint32_t a, const double* dist, int nmoving, int species, ora_drecord* rec) {
    attempt = a;
    uidx = 0;
    npair = 0;
    ora_drecord dummy;
    if (!rec) rec = &dummy;
    memset(rec, 0, sizeof(*rec));
    std::vector<int> idx(nmoving);
    for (int im = 0; im < nmoving;) {
      int i;
      if (species < 0) {
        i = (int)(np * uniform());
        if (i == np) continue;
      } else {
        const int nsp = cfg.spec_count[species], f = spec_first[species];
        i = (int)(nsp * uniform() + f);
        if (i == nsp + f) i = nsp + f - 1;
      }
      bool dup = false;
      for (int jm = 0; jm < im; ++jm) dup |= idx[jm] == i;
      if (!dup) idx[im++] = i;
    }
    std::vector<V3> disp(nmoving);
    for (int k = 0; k < nmoving; ++k)
      for (int d = 0; d < 3; ++d) disp[k].x[d] = uniform();
    for (int k = 0; k < nmoving; ++k)
      for (int d = 0; d < 3; ++d) {
        disp[k].x[d] -= 0.5;
        disp[k].x[d] *= dist[d];
      }
    const int i1 = 0, i2 = fixed_node ? ns / 2 - 1 : ns - 1;
    double ds = actionDisplaceDiff(idx, disp, i1, i2);
    if (fixed_node) ds += actionDisplaceDiff(idx, disp, i1 + ns / 2, i2 + ns / 2);
    double dsn = 0;
    if (fixed_node)
      for (int sp = 0; sp < cfg.nspecies; ++sp)
        if (nodes[sp].kind) dsn += nodeDisplaceDiff(sp, idx, disp, i1, i2);
    for (int k = 0; k < nmoving && k < ORA_MAX_MOVING; ++k) {
      rec->ipart[k] = idx[k];
      for (int d = 0; d < 3; ++d) rec->disp[k][d] = disp[k].x[d];
    }
    rec->ds = ds;
    rec->ds_node = dsn;
    const double acceptProb = exp(-(ds + dsn) + 0.0);
    if (uniform() > acceptProb) return false;
    rec->accepted = 1;
    for (int t = i1; t <= i2; ++t)
      for (int k = 0; k < nmoving; ++k) {
        for (int half = 0; half < (fixed_node ? 2 : 1); ++half) {
          V3& b = P(t + half * (ns / 2), idx[k]);
          for (int d = 0; d < 3; ++d) b.x[d] += disp[k].x[d];
          cell.pbc(b.x);
        }
      }
    return true;
  }
};

}  // namespace

extern "C" {

double port_virial_energy(void* h, int nwindow);
int port_run_displace(void* h, int n, uint32_t first_attempt, const double* dist, int nmoving,
                      int species, ora_drecord* recs);
double port_coulomb_energy(void* h, double epsilon);
double port_ewald_coulomb_energy(void* h, double epsilon, double rcut, const ora_ewald_table* est,
                                 const double* vgrid);

void* port_create(const ora_config* c, int npair_tables, const int* pair_species,
                  const ora_pair_table* tables, const ora_ewald_table* ew) {
  Sim* s = new Sim();
  s->cfg = *c;
  s->np = c->npart;
  s->ns = c->nslice;
  s->L = c->nlevel;
  s->nsec = (1 << c->nlevel) + 1;
  s->cell.init(c->cell);
  int first = 0;
  s->spec_first.resize(c->nspecies);
  for (int sp = 0; sp < c->nspecies; ++sp) {
    s->spec_first[sp] = first;
    for (int k = 0; k < c->spec_count[sp]; ++k) {
      s->spec.push_back(sp);
      s->lambda.push_back(0.5 / c->spec_mass[sp]);
    }
    first += c->spec_count[sp];
  }
  s->path.assign((size_t)s->ns * s->np, V3());
  s->sec1.assign((size_t)s->nsec * s->np, V3());
  s->sec2.assign((size_t)s->nsec * s->np, V3());
  s->mov1.assign(s->nsec, V3());
  for (int k = 0; k < npair_tables; ++k) {
    PairTab pt;
    pt.s1 = pair_species[2 * k];
    pt.s2 = pair_species[2 * k + 1];
    pt.ifirst1 = s->spec_first[pt.s1];
    pt.npart1 = c->spec_count[pt.s1];
    pt.ifirst2 = s->spec_first[pt.s2];
    pt.npart2 = c->spec_count[pt.s2];
    pt.ngpts = tables[k].ngpts;
    pt.norder = tables[k].norder;
    pt.ndata = pt.norder + 1;
    pt.rgridinv = tables[k].rgridinv;
    pt.logrratioinv = tables[k].logrratioinv;
    pt.ugrid.assign(tables[k].ugrid, tables[k].ugrid + (size_t)pt.ngpts * 2 * pt.ndata);
    s->pairs.push_back(pt);
  }
  if (ew && c->ewald) {
    s->has_ewald = true;
    s->ewald.totk = ew->totk;
    s->ewald.kvec.assign(ew->kvec, ew->kvec + 3 * ew->totk);
    s->ewald.vk.assign(ew->vk, ew->vk + ew->totk);
    s->ewald.oneOver2V = ew->one_over_2v;
    s->ewald.selfEnergy = ew->self_energy;
    for (int d = 0; d < 3; ++d) {
      s->ewald.ikmax[d] = ew->ikmax[d];
      s->ewald.deltak[d] = 2 * 3.14159265358979 * s->cell.b[d];
    }
    for (int p = 0; p < s->np; ++p) s->ewald.q.push_back(c->spec_charge[s->spec[p]]);
  }
  // Periodic Gaussians as SpringAction / FreeMover(PBC) build them.
  const int nsp = c->nspecies;
  s->pg_spring.assign((c->nlevel + 1) * nsp * 3, PGauss());
  s->has_pg_spring.assign((c->nlevel + 1) * nsp * 3, 0);
  s->pg_mover.assign((c->nlevel + 2) * nsp * 3, PGauss());
  s->has_pg_mover.assign((c->nlevel + 2) * nsp * 3, 0);
  for (int lev = 0; lev <= c->nlevel + 1; ++lev)
    for (int sp = 0; sp < nsp; ++sp)
      for (int d = 0; d < 3; ++d) {
        const int k = (lev * nsp + sp) * 3 + d;
        if (lev <= c->nlevel) {
          double alpha = c->spec_mass[sp] / (2 * c->tau * (1 << lev));
          if (PGauss::numberOfTerms(alpha, c->cell[d]) < 16) {
            s->pg_spring[k].init(alpha, c->cell[d]);
            s->has_pg_spring[k] = 1;
          }
        }
        // FreeMover builds levels 0..nlevel, FreeMoverPBC 0..nlevel+1.
        if (lev <= c->nlevel || c->mover == 1) {
          double alpha = c->spec_mass[sp] / (c->tau * (1 << lev));
          if (PGauss::numberOfTerms(alpha, c->cell[d]) < 16) {
            s->pg_mover[k].init(alpha, c->cell[d]);
            s->has_pg_mover[k] = 1;
          }
        }
      }
  s->nodes.resize(nsp);
  s->fn.resize(nsp);
  for (int sp = 0; sp < nsp; ++sp) {
    NodeModel& nm = s->nodes[sp];
    nm.kind = c->node_kind[sp];
    if (!nm.kind) continue;
    s->fixed_node = true;
    nm.npart = c->spec_count[sp];
    nm.ifirst = s->spec_first[sp];
    nm.tau = c->tau;
    nm.mass = c->spec_mass[sp];
    nm.omega = c->node_omega[sp];
    nm.temperature = c->node_temperature;
    nm.cell = &s->cell;
    if (nm.kind == 1) {
      nm.coshwt = cosh(nm.omega * 0.5 / nm.temperature);
      nm.sinhwt = sinh(nm.omega * 0.5 / nm.temperature);
      nm.c = nm.mass * 0.5 * nm.omega / nm.sinhwt;
    } else {
      for (int d = 0; d < 3; ++d) nm.pg[d].init(nm.mass * nm.temperature, c->cell[d]);
    }
    nm.matrix.assign((size_t)s->nsec * nm.npart * nm.npart, 0.0);
    Sim::FNState& st = s->fn[sp];
    st.dm.assign(s->nsec, 0.0);
    st.newdm.assign(s->nsec, 0.0);
    st.dist.assign((size_t)s->nsec * 2 * s->np, 0.0);
    st.newdist.assign((size_t)s->nsec * 2 * s->np, 0.0);
    st.notMySpecies = false;
  }
  s->nerror_init = 0;
  return s;
}

void port_destroy(void* h) { delete (Sim*)h; }

void port_set_path(void* h, const double* xyz) {
  Sim* s = (Sim*)h;
  memcpy(s->path.data(), xyz, sizeof(double) * 3 * s->np * s->ns);
}

void port_get_path(void* h, double* xyz) {
  Sim* s = (Sim*)h;
  memcpy(xyz, s->path.data(), sizeof(double) * 3 * s->np * s->ns);
}

int port_run(void* h, int n, uint32_t first_attempt, ora_record* recs) {
  Sim* s = (Sim*)h;
  int nacc = 0;
  for (int a = 0; a < n; ++a)
    if (s->attemptMove(first_attempt + (uint32_t)a, recs ? &recs[a] : 0)) ++nacc;
  return nacc;
}

double port_thermo_energy(void* h) { return ((Sim*)h)->thermoEnergy(); }
int port_run_displace(void* h, int n, uint32_t first_attempt, const double* dist, int nmoving,
                      int species, ora_drecord* recs) {
  Sim* s = (Sim*)h;
  int nacc = 0;
  for (int a = 0; a < n; ++a)
    nacc += s->displaceMove(first_attempt + (uint32_t)a, dist, nmoving, species,
                            recs ? &recs[a] : nullptr);
  return nacc;
}
double port_virial_energy(void* h, int nwindow) { return ((Sim*)h)->virialEnergy(nwindow); }
double port_coulomb_energy(void* h, double epsilon) { return ((Sim*)h)->coulombEnergy(epsilon); }
double port_ewald_coulomb_energy(void* h, double epsilon, double rcut, const ora_ewald_table* est,
                                 const double* vgrid) {
  Sim* s = (Sim*)h;
  Ewald E;
  E.totk = est->totk;
  E.kvec.assign(est->kvec, est->kvec + 3 * est->totk);
  E.vk.assign(est->vk, est->vk + est->totk);
  E.oneOver2V = est->one_over_2v;
  E.selfEnergy = est->self_energy;
  for (int d = 0; d < 3; ++d) {
    E.ikmax[d] = est->ikmax[d];
    E.deltak[d] = 2 * 3.14159265358979 * s->cell.b[d];
  }
  for (int i = 0; i < s->np; ++i) E.q.push_back(s->charge(i));
  std::vector<double> vg(vgrid, vgrid + 1001);
  return s->ewaldCoulombEnergy(epsilon, rcut, E, vg);
}

double port_bead_utau(void* h, int ipart, int islice) {
  return ((Sim*)h)->beadUtau(ipart, islice);
}

double port_action_diff(void* h, int level, const double* section, const double* moving,
                        int ipart) {
  Sim* s = (Sim*)h;
  std::vector<V3> sec((size_t)s->nsec * s->np), mov(s->nsec);
  memcpy(sec.data(), section, sizeof(double) * 3 * s->nsec * s->np);
  memcpy(mov.data(), moving, sizeof(double) * 3 * s->nsec);
  return s->actionDiff(sec, mov, ipart, level);
}

int port_node_eval(void* h, int sp, const double* r1, const double* r2, int islice,
                   int scale_magnitude, double* det, double* d1, double* d2) {
  Sim* s = (Sim*)h;
  if (!s->nodes[sp].kind) return -1;
  std::vector<V3> a1(s->np), a2(s->np);
  memcpy(a1.data(), r1, sizeof(double) * 3 * s->np);
  memcpy(a2.data(), r2, sizeof(double) * 3 * s->np);
  int err = s->nodes[sp].evaluate(a1, a2, islice, scale_magnitude != 0, det);
  s->nodes[sp].distance(a1, a2, islice, d1, d2, s->np);
  return err;
}

double port_node_scale(void* h, int sp) { return ((Sim*)h)->nodes[sp].scale; }
void port_set_node_scale(void* h, int sp, double v) { ((Sim*)h)->nodes[sp].scale = v; }
int port_init_errors(void* h) { return ((Sim*)h)->nerror_init; }

double port_ewald_long_range(void* h, const double* r) {
  Sim* s = (Sim*)h;
  std::vector<V3> rv(s->np);
  memcpy(rv.data(), r, sizeof(double) * 3 * s->np);
  return s->ewald.evalLongRange(rv);
}

// The replayed random streams (CPU side of the bit-exactness check).
void port_stream_sample(uint64_t seed, uint32_t replica, uint32_t attempt, int n, double* u,
                        double* z) {
  for (int i = 0; i < n; ++i) {
    u[i] = pimc::stream_uniform(seed, replica, attempt, (uint32_t)i);
    z[i] = pimc::stream_normal(seed, replica, attempt, (uint32_t)i);
  }
}

// Pieces exposed for the reference unit-test known answers.
int port_pg_terms(double alpha, double length) { return PGauss::numberOfTerms(alpha, length); }
double port_pg_eval(double alpha, double length, double x, double* grad) {
  PGauss g;
  g.init(alpha, length);
  double v = g.evaluate(x);
  *grad = g.gradient;
  return v;
}
void port_pbc(const double* a, double* v) {
  Cell c;
  c.init(a);
  c.pbc(v);
}

}  // extern "C"
