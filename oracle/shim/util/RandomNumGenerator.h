/* Replay shim for pi-qmc's RandomNumGenerator (src/util/RandomNumGenerator.h:23-87).
   Same class and method names, so the reference sources compile unchanged; the
   numbers come from the engine's counter-based streams (pimc_rng.h) through
   oracle_shim_uniform()/oracle_shim_normals(), in pi-qmc's consumption order.
   makeGaussRand keeps the reference's pairing: n normals take ceil(n/2)
   Box-Muller pairs and an odd tail uses only the cosine leg. */
#ifndef __RandomNumGenerator_h_
#define __RandomNumGenerator_h_
#include "config.h"
#include <cstdlib>
#include <cmath>
#include <blitz/array.h>

extern "C" double oracle_shim_uniform(void);
extern "C" void oracle_shim_normals(double* out, int n);

class RandomNumGenerator {
public:
  static void seed(const int) {}
  static double getRand() { return oracle_shim_uniform(); }
  static void makeRand(blitz::Array<double, 1>& a) {
    for (int i = 0; i < a.size(); ++i) a(i) = getRand();
  }
  template <int N>
  static void makeRand(blitz::Array<blitz::TinyVector<double, N>, 1>& a) {
    for (int j = 0; j < a.size(); ++j)
      for (int i = 0; i < N; ++i) a(j)[i] = getRand();
  }
  static void makeGaussRand(blitz::Array<double, 1>& a) {
    oracle_shim_normals((double*)&a(0), a.size());
  }
  template <int TDIM>
  static void makeGaussRand(blitz::Array<blitz::TinyVector<double, TDIM>, 1>& a) {
    oracle_shim_normals((double*)&a(0), TDIM * a.size());
  }
};
#endif
