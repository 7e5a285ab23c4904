// Host-side construction of the read-only tables the kernels consume:
//  * the tabulated Coulomb pair action of every interacting species pair
//    (what CoulombAction's constructor builds, src/action/CoulombAction.cc:19-91,
//    PairAction's empirical-action constructor, src/action/PairAction.cc:161-185,
//    from the Coulomb link-action fit, src/action/coulomb/*.cpp), and
//  * the optimised Ewald split (OptEwaldSum, src/util/OptEwaldSum.cc:28-245) with
//    its half-space k-vector list (EwaldSum, src/util/EwaldSum.cc:16-90).
// The fit coefficients below are pi-qmc's published Coulomb link-action fit; the
// engine reproduces pi-qmc's tables so that an engine built standalone samples
// the same pair action pi-qmc would.
#include <cmath>
#include <complex>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/pimc_gb300.h"

namespace {

// Horner evaluation c0 + x (c1 + x (c2 + ...)).
double horner(const double* c, int n, double x) {
  double v = c[n - 1];
  for (int i = n - 2; i >= 0; --i) v = c[i] + x * v;
  return v;
}

// One-dimensional Coulomb link action as a function of reff = 2 mu q1q2 r for a
// given stau = q1q2 sqrt(2 mu tau): value at the origin and the s-expansion
// terms u0..u4 as rational fits.
struct Link1D {
  double st, i1, i2, i3, i4, i5;
  explicit Link1D(double stau) : st(stau) {
    i1 = 1.0 / st;
    i2 = i1 * i1;
    i3 = i2 * i1;
    i4 = i3 * i1;
    i5 = i4 * i1;
  }
  double origin() const {
    static const double c[] = {1.772453851, -0.074137740, 0.005834805, -0.000382686,
                               0.000008738, 0.000002138};
    return st * horner(c, 6, st);
  }
  double u0(double uo, double x) const {
    const double a = 0.25300593 * i1 + 0.01432126;
    const double b = 0.07936898 * i2 - 0.01634421 / st;
    const double c = 0.07263383 * i3, d = 0.00940013 * i4, e = 0.03160181 * i5;
    const double f = 0.18976335 * i1, g = 0.00343053 * i2;
    const double num = uo + x * ((uo * a - 1.) + x * (f + x * (g + x * e * st * st)));
    return num / (1. + x * (a + x * (b + x * (c + x * (d + x * e)))));
  }
  double u1(double x) const {
    const double num[] = {0.07776906 * i1, -0.04695226 * i2, 0.01291994 * i3};
    const double den[] = {1.0, 0.60942687 * i1, -1.09588064 * i2, 1.15591565 * i3,
                          -0.57485278 * i4, 0.15212765 * i5};
    return x * x * horner(num, 3, x) / horner(den, 6, x);
  }
  double u2(double x) const {
    const double num[] = {9.52130652e-04 * i3, -6.39946071e-04 * i4, 1.14359558e-04 * i5};
    const double den[] = {-7.59575215e-01 * i3, 5.53798980e-01 * i4, -7.15626226e-02 * i5,
                          -3.49081618e-02 * i5 * i1, 8.40084881e-03 * i5 * i2};
    return std::pow(x, 4) * horner(num, 3, x) / (1 + std::pow(x, 3) * horner(den, 5, x));
  }
  double u3(double x) const {
    const double num[] = {-2.06984256e-1 * i5, -9.51423947e-3 * i5 * i1, 8.97532561e-2 * i5 * i2};
    const double den[] = {6.10876797e+4 * i3,      -1.19016292e+5 * i4,      9.29836599e+4 * i5,
                          -3.49919130e+4 * i5 * i1, 6.42490539e+3 * i5 * i2, -6.02729064e+2 * i5 * i3,
                          6.01285550e+1 * i5 * i4};
    return std::pow(x, 6) * horner(num, 3, x) / (1 + std::pow(x, 3) * horner(den, 7, x));
  }
  double u4(double x) const {
    const double a = -2.84102296e-6 * i5, b = 6.26961672e-7 * i5 * i2;
    const double den[] = {-2.20166473e-1 * i3, 1.07981903e-1 * i5, -1.94671111e-2 * i5 * i2,
                          1.56217930e-3 * i5 * i4};
    return std::pow(x, 6) * (a + b * x * x) / (1 + x * x * x * horner(den, 4, x * x));
  }
};

// Three-dimensional link-action terms extracted from the 1-D fit
// (the k-th coefficient of the off-diagonal s^2 expansion).
double link3d(const Link1D& c, int order, double x) {
  const double st = c.st;
  if (order == 0 || order == 1) {
    const double g1 = c.u1(x);
    const double a = 0.5 * x * x / (st * st);
    const double b = std::exp(-2. * a);
    const double cc = 1.0 / (1.0 + 2 * (1.0 - b) * g1 / (a + 1e-200));
    if (order == 0) return c.u0(c.origin(), x) + std::log(cc);
    return g1 + cc * (b * g1 - 4 * (1 - b) * c.u2(x) / (a + 1e-200));
  }
  if (order == 4) return c.u4(x);
  const double g1 = c.u1(x), g2 = c.u2(x), g3 = c.u3(x);
  const double a = 2. * st * st / (x * x + 1e-50);
  const double b = std::exp(-2. / (a + 1e-200));
  const double cc = 1. / (1 + 2 * a * (1 - b) * g1);
  if (order == 2) {
    return g2 + 0.25 * cc / (a + 1e-200) *
                    (cc * (b * g1 * (1 + 2 * a * g1) + 8 * a * b * g2 +
                           32 * a * a * a * (1 - b) * (1 - b) * g2 * g2) -
                     24 * a * a * (1 - b) * g3);
  }
  const double g4 = c.u4(x);
  const double a2 = a * a, a3 = a2 * a, a4 = a3 * a, a5 = a4 * a;
  const double p = 1 + 2 * a * g1;
  const double t1 = 128 * a5 * b * b * b * (4 * g2 * g2 * g2 - 9 * g1 * g2 * g3 + 6 * g1 * g1 * g4);
  const double t2 = 64 * a3 * (a * g2 * (-8 * a * g2 * g2 + 9 * p * g3) - 3 * p * p * g4);
  const double t3 =
      2 * a * b * b *
      (2 * a * g1 * g1 * g1 + 96 * a2 * g2 * (g2 - 8 * a2 * g2 * g2 + 3 * a * g3) +
       12 * a * g1 * (g2 - 6 * a * g3 + 144 * a3 * g2 * g3 - 32 * a2 * g4) +
       g1 * g1 * (1 - 1152 * a4 * g4));
  const double t4 =
      b * (4 * a2 * g1 * g1 * g1 +
           12 * a * (g2 - 16 * a2 * g2 * g2 + 128 * a4 * g2 * g2 * g2 + 6 * a * g3 -
                     96 * a3 * g2 * g3 + 16 * a2 * g4) +
           4 * g1 * g1 * (a + 576 * a5 * g4) +
           g1 * (1 + 24 * a2 * (g2 + 6 * a * g3 - 144 * a3 * g2 * g3 + 64 * a2 * g4)));
  return g3 + cc * cc * cc / (24. * a2 + 1e-200) * (t1 + t2 + t3 + t4);
}

const double kEwaldPi = 3.14159265358979;  // the value EwaldSum uses

struct OptEwald {
  double rcut = 0, kcut = 0, oneOver2V = 0, selfEnergy = 0;
  int npoly = 8;
  std::vector<double> coef;
  std::vector<int> kvec;
  std::vector<double> vk;
  int ikmax[3] = {0, 0, 0};

  double evalFR(double r) const {
    if (r > rcut) return 1. / r;
    double v = 0, r2 = r * r;
    for (int i = npoly - 1; i >= 0; --i) v = v * r2 + coef[i];
    return v;
  }
  double evalFRcut(const std::vector<double>& t, int nd) const {
    double v = 0;
    for (int i = 0; i < npoly; ++i) {
      double x = std::pow(rcut, 2 * i - nd);
      for (int j = 0; j < nd; ++j) x *= 2 * i - j;
      v += t[i] * x;
    }
    return v;
  }
  // Fourier transform of the short-range basis r^(2n) on [0, rcut] by the
  // recurrence temp_n = (rcut^(n+1) e^{ik rcut} - (n+1) temp_{n-1}) / (ik).
  void basis_ft(double k, std::vector<double>& ft, double& v1r) const {
    typedef std::complex<double> Z;
    const Z eikr = std::exp(Z(0., k * rcut));
    Z temp = (eikr - 1.) / Z(0., k);
    v1r = 4. * kEwaldPi * std::imag(temp) / k;
    double rn = rcut;
    for (int n = 0; n < 2 * npoly - 1; ++n) {
      temp = (rn * eikr - (n + 1.) * temp) / Z(0., k);
      rn *= rcut;
      if (n % 2 == 0) ft[n / 2] = 4. * kEwaldPi * std::imag(temp) / k;
    }
  }
  double evalFK(double k) const {
    std::vector<double> ft(npoly);
    double v1r;
    basis_ft(k, ft, v1r);
    double v = 4. * kEwaldPi / (k * k) - v1r;
    for (int i = 0; i < npoly; ++i) v += coef[i] * ft[i];
    return v;
  }
  double evalFK0() const {
    double fn = 2. * kEwaldPi * rcut * rcut;
    double v = -fn;
    fn *= rcut / 3.;
    for (int n = 0; n < 2 * npoly; n += 2) {
      v += coef[n / 2] * fn;
      fn *= (rcut * rcut) * (n + 3.) / (n + 5.);
    }
    return v;
  }
};

// Solves a x = b (n x n, column-major a overwritten) by Gaussian elimination
// with partial pivoting.
bool solve(std::vector<double> a, int n, std::vector<double>& b) {
  std::vector<int> piv(n);
  for (int j = 0; j < n; ++j) {
    int p = j;
    for (int i = j + 1; i < n; ++i)
      if (std::fabs(a[i + j * n]) > std::fabs(a[p + j * n])) p = i;
    if (a[p + j * n] == 0.0) return false;
    if (p != j) {
      for (int k = 0; k < n; ++k) std::swap(a[j + k * n], a[p + k * n]);
      std::swap(b[j], b[p]);
    }
    for (int i = j + 1; i < n; ++i) {
      const double l = a[i + j * n] / a[j + j * n];
      for (int k = j + 1; k < n; ++k) a[i + k * n] -= l * a[j + k * n];
      b[i] -= l * b[j];
    }
  }
  for (int j = n - 1; j >= 0; --j) {
    for (int k = j + 1; k < n; ++k) b[j] -= a[j + k * n] * b[k];
    b[j] /= a[j + j * n];
  }
  return true;
}

bool build_opt_ewald(const double* cell, const double* q, int npart, double rcut, double kcut,
                     OptEwald& E) {
  E = OptEwald();
  E.rcut = rcut;
  E.kcut = kcut;
  const int np = E.npoly;
  const double khalo = 4 * kcut, kcut2 = kcut * kcut, khalo2 = khalo * khalo;
  double dk[3], dk2[3];
  for (int i = 0; i < 3; ++i) {
    dk[i] = 2 * kEwaldPi / cell[i];
    dk2[i] = dk[i] * dk[i];
  }
  // k values in the halo kcut < |k| < khalo with their degeneracies (one octant).
  std::vector<double> kval;
  std::vector<int> degen;
  for (int i = 0; i < khalo / dk[0]; ++i) {
    const double kx2 = i * i * dk2[0];
    const int gx = (i == 0) ? 1 : 2;
    for (int j = 0; j < std::sqrt(khalo2 - kx2) / dk[1]; ++j) {
      const double kxy2 = kx2 + j * j * dk2[1];
      const int gxy = gx * ((j == 0) ? 1 : 2);
      for (int k = 0; k < std::sqrt(khalo2 - kxy2) / dk[2]; ++k) {
        const double k2 = kxy2 + k * k * dk2[2];
        if (k2 > kcut2) {
          kval.push_back(std::sqrt(k2));
          degen.push_back(gxy * ((k == 0) ? 1 : 2));
        }
      }
    }
  }
  // Least squares for the short-range polynomial against the bare 1/r in the
  // halo, with the value and slope of 1/r imposed at rcut.  pi-qmc forms the
  // normal equations in the monomial basis r^(2n) (condition number ~1e32 for
  // rcut ~ 12) and adds the constraints by Lagrange multipliers; here the same
  // problem is solved as one KKT system in the scaled basis (r/rcut)^(2n), where
  // it is well determined.
  std::vector<double> ft(np), scale(np);
  for (int i = 0; i < np; ++i) scale[i] = std::pow(rcut, 2 * i);
  const int nk = np + 2;
  std::vector<double> K(nk * nk, 0.0), rhs(nk, 0.0);
  for (size_t ik = 0; ik < kval.size(); ++ik) {
    const double k = kval[ik];
    double v1r;
    E.basis_ft(k, ft, v1r);
    const double v = -4. * kEwaldPi / (k * k) + v1r;
    for (int i = 0; i < np; ++i) {
      const double gi = ft[i] / scale[i];
      rhs[i] += degen[ik] * v * gi;
      for (int j = 0; j < np; ++j) K[i + j * nk] += degen[ik] * gi * (ft[j] / scale[j]);
    }
  }
  for (int i = 0; i < np; ++i) {
    const double ci = 1.0;              // (r/rcut)^(2i) at r = rcut
    const double di = (2.0 * i) / rcut;  // its derivative
    K[i + np * nk] = K[np + i * nk] = ci;
    K[i + (np + 1) * nk] = K[(np + 1) + i * nk] = di;
  }
  rhs[np] = 1. / rcut;
  rhs[np + 1] = -1. / (rcut * rcut);
  if (!solve(K, nk, rhs)) return false;
  E.coef.assign(np, 0.0);
  for (int i = 0; i < np; ++i) E.coef[i] = rhs[i] / scale[i];
  // Half-space k-vectors with 0 < |k| < kcut (strict), as EwaldSum enumerates them.
  for (int i = 0; i < 3; ++i) E.ikmax[i] = (int)(cell[i] * kcut / (2 * kEwaldPi));
  const double dkr[3] = {2 * kEwaldPi / cell[0], 2 * kEwaldPi / cell[1], 2 * kEwaldPi / cell[2]};
  for (int kx = 0; kx <= E.ikmax[0]; ++kx) {
    const double kx2 = kx * kx * dkr[0] * dkr[0];
    for (int ky = (kx == 0 ? 0 : -E.ikmax[1]); ky <= E.ikmax[1]; ++ky) {
      const double ky2 = ky * ky * dkr[1] * dkr[1];
      for (int kz = ((kx == 0 && ky == 0) ? 0 : -E.ikmax[2]); kz <= E.ikmax[2]; ++kz) {
        const double k2 = kx2 + ky2 + kz * kz * dkr[2] * dkr[2];
        if (k2 < kcut * kcut && k2 != 0) {
          E.kvec.push_back(kx);
          E.kvec.push_back(ky);
          E.kvec.push_back(kz);
          E.vk.push_back(E.evalFK(std::sqrt(k2)));
        }
      }
    }
  }
  E.oneOver2V = 0.5 / (cell[0] * cell[1] * cell[2]);
  double Q = 0, Q2 = 0;
  for (int i = 0; i < npart; ++i) {
    Q += q[i];
    Q2 += q[i] * q[i];
  }
  E.selfEnergy = -0.5 * Q2 * E.coef[0] + E.oneOver2V * E.evalFK0() * Q * Q;
  return true;
}

struct CoulombTables {
  std::vector<std::vector<double>> grids;
  std::vector<pimc_pair_table> tabs;
  OptEwald ewald;
  bool has_ewald = false;
};

thread_local CoulombTables g_tables;
thread_local std::string g_table_err;

}  // namespace

extern "C" {

// Builds the CoulombAction tables for `sys` (species pairs i <= j with nonzero
// charge product and either distinct species or more than one particle, in
// that order) and, when sys->ewald, the OptEwaldSum long-range table with real-
// space cutoff rcut (0: half the first box side) and k cutoff kcut.  rmin/rmax
// of the log grid default as in pi-qmc (0.005/(2 mu |q1q2|) and the cell
// diagonal); ngpts defaults to 500.  The returned arrays stay valid until the
// next call on the same thread.
int pimc_coulomb_tables(const pimc_system* sys, int norder, int ngpts, double rmin, double rmax,
                        double ewald_rcut, double ewald_kcut, const pimc_pair_table** tables,
                        int* ntables, const pimc_ewald_table** ewald) {
  if (!sys || !tables || !ntables) return PIMC_ERR_INVALID;
  CoulombTables& T = g_tables;
  T.grids.clear();
  T.tabs.clear();
  T.has_ewald = false;
  const double tau = sys->tau, eps = sys->epsilon > 0 ? sys->epsilon : 1.0;
  std::vector<double> q;
  for (int s = 0; s < sys->nspecies; ++s)
    for (int k = 0; k < sys->spec_count[s]; ++k) q.push_back(sys->spec_charge[s]);
  if (sys->ewald) {
    if (ewald_rcut == 0.) ewald_rcut = sys->cell[0] / 2.;
    if (!build_opt_ewald(sys->cell, q.data(), sys->npart, ewald_rcut, ewald_kcut, T.ewald))
      return PIMC_ERR_INVALID;
    T.has_ewald = true;
  }
  if (ngpts == 0) ngpts = 500;
  for (int i = 0; i < sys->nspecies; ++i) {
    for (int j = i; j < sys->nspecies; ++j) {
      const double q1q2 = sys->spec_charge[i] * sys->spec_charge[j] / eps;
      if (!(q1q2 != 0 && (i != j || sys->spec_count[i] > 1))) continue;
      const double mu = 1. / (1. / sys->spec_mass[i] + 1. / sys->spec_mass[j]);
      if (rmin == 0) rmin = 0.005 / (2 * ((mu > 500) ? 1 : mu) * std::fabs(q1q2));
      if (rmax == 0)
        rmax = std::sqrt(sys->cell[0] * sys->cell[0] + sys->cell[1] * sys->cell[1] +
                         sys->cell[2] * sys->cell[2]);
      const int no = (mu > 500) ? 0 : norder;
      const double rgridinv = 1.0 / rmin, logrratioinv = (ngpts - 1) / std::log(rmax / rmin);
      std::vector<double> g((size_t)ngpts * 2 * (no + 1), 0.0);
      auto u = [&](double r, int order, double t) {
        r = std::sqrt(r * r + 0.0);
        const double reff = 2.0 * mu * q1q2 * r;
        const Link1D c(q1q2 * std::sqrt(2.0 * mu * t));
        double v = link3d(c, order, reff);
        if (order == 0 && T.has_ewald) v -= t * q1q2 * T.ewald.evalFR(r);
        return v;
      };
      for (int k = 0; k < ngpts; ++k) {
        const double r = (1. / rgridinv) * std::exp(k / logrratioinv);
        for (int o = 0; o <= no; ++o) {
          g[(k * 2 + 0) * (no + 1) + o] = u(r, o, tau);
          // tau derivative by central difference, as CoulombAction::utau
          const double e = 1e-7;
          const double up = u(r, o, tau * (1.0 + e)), um = u(r, o, tau * (1.0 - e));
          g[(k * 2 + 1) * (no + 1) + o] = (up - um) / (2.0 * e * tau);
        }
      }
      T.grids.push_back(std::move(g));
      pimc_pair_table pt;
      pt.species1 = i;
      pt.species2 = j;
      pt.ngpts = ngpts;
      pt.norder = no;
      pt.rgridinv = rgridinv;
      pt.logrratioinv = logrratioinv;
      pt.ugrid = nullptr;
      T.tabs.push_back(pt);
    }
  }
  for (size_t k = 0; k < T.tabs.size(); ++k) T.tabs[k].ugrid = T.grids[k].data();
  *tables = T.tabs.data();
  *ntables = (int)T.tabs.size();
  if (ewald) {
    static thread_local pimc_ewald_table et;
    if (T.has_ewald) {
      et.totk = (int)T.ewald.vk.size();
      et.kvec = T.ewald.kvec.data();
      et.vk = T.ewald.vk.data();
      et.one_over_2v = T.ewald.oneOver2V;
      et.self_energy = T.ewald.selfEnergy;
      for (int a = 0; a < 3; ++a) et.ikmax[a] = T.ewald.ikmax[a];
      *ewald = &et;
    } else {
      *ewald = nullptr;
    }
  }
  return PIMC_OK;
}

// The optimized Ewald sum an EwaldCoulombEstimator builds for itself
// (src/estimator/EwaldCoulombEstimator.cc:60-90, the same fit as the action's with
// the estimator's rcut and kcut): its k-list table and the 1001-point grid
// vgrid[i] = -f(i rcut/1000)/epsilon (vgrid[0] = -f(0)/epsilon).  The table stays
// valid until the next call on the same thread.
int pimc_ewald_estimator_tables(const pimc_system* sys, double rcut, double kcut, double epsilon,
                                const pimc_ewald_table** est, double* vgrid) {
  if (!sys || !est || !vgrid || !(rcut > 0) || !(kcut > 0) || !(epsilon > 0))
    return PIMC_ERR_INVALID;
  static thread_local OptEwald E;
  static thread_local pimc_ewald_table et;
  std::vector<double> q;
  for (int s = 0; s < sys->nspecies; ++s)
    for (int k = 0; k < sys->spec_count[s]; ++k) q.push_back(sys->spec_charge[s]);
  if (!build_opt_ewald(sys->cell, q.data(), sys->npart, rcut, kcut, E)) return PIMC_ERR_INVALID;
  const double dr = rcut / 1000;
  vgrid[0] = -E.coef[0] / epsilon;
  for (int i = 1; i < 1001; ++i) vgrid[i] = -E.evalFR(i * dr) / epsilon;
  et.totk = (int)E.vk.size();
  et.kvec = E.kvec.data();
  et.vk = E.vk.data();
  et.one_over_2v = E.oneOver2V;
  et.self_energy = E.selfEnergy;
  for (int a = 0; a < 3; ++a) et.ikmax[a] = E.ikmax[a];
  *est = &et;
  return PIMC_OK;
}

// The short-range polynomial coefficients of the last Ewald table built.
int pimc_ewald_coefficients(double* coef, int n) {
  if (!g_tables.has_ewald) return PIMC_ERR_INVALID;
  for (int i = 0; i < n && i < (int)g_tables.ewald.coef.size(); ++i) coef[i] = g_tables.ewald.coef[i];
  return PIMC_OK;
}

}  // extern "C"
