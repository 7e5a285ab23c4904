// Counter-based random streams for the bisection sampler.
//
// pi-qmc draws uniforms from libc rand() and normals from a Box-Muller pair
// (src/util/RandomNumGenerator.h:41-85).  A sequential global stream cannot be
// shared by thousands of replicas advancing in one launch, so this engine uses
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11) keyed by the run seed and
// addressed by (replica, attempt, index).  Every random number consumed in one
// section-move attempt has a fixed address, in the order pi-qmc consumes them:
//
//   uniform j of attempt a of replica r : ctr = {j/2, a, r, 0}, words 2(j%2), 2(j%2)+1
//   normal  k of attempt a of replica r : ctr = {k/2, a, r, 1}, Box-Muller of the two
//                                         53-bit uniforms in that block; k even = cos leg
//
// The normal transform is built only from correctly rounded IEEE-754 operations
// (add, mul, fma, div, sqrt) with every rounding written out, so host code built
// with -ffp-contract=off and device code produce bit-identical normals.  That is
// what lets the CPU oracle replay exactly the proposals a kernel made.
// log() is the atanh series log(m) = 2 atanh((m-1)/(m+1)) (Abramowitz & Stegun
// 4.1.27) after an exact power-of-two split; sin/cos are Taylor series after an
// exact quarter-turn reduction of the uniform itself.
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define PIMC_HD __host__ __device__ __forceinline__
#else
#define PIMC_HD static inline
#endif

#if defined(__CUDA_ARCH__)
#define PR_ADD(a, b) __dadd_rn((a), (b))
#define PR_SUB(a, b) __dsub_rn((a), (b))
#define PR_MUL(a, b) __dmul_rn((a), (b))
#define PR_FMA(a, b, c) __fma_rn((a), (b), (c))
#define PR_DIV(a, b) __ddiv_rn((a), (b))
#define PR_SQRT(a) __dsqrt_rn(a)
#else
#include <math.h>
#define PR_ADD(a, b) ((a) + (b))
#define PR_SUB(a, b) ((a) - (b))
#define PR_MUL(a, b) ((a) * (b))
#define PR_FMA(a, b, c) fma((a), (b), (c))
#define PR_DIV(a, b) ((a) / (b))
#define PR_SQRT(a) sqrt(a)
#endif

namespace pimc {

struct Philox4 {
  uint32_t v[4];
};

PIMC_HD uint32_t mulhi32(uint32_t a, uint32_t b) {
#if defined(__CUDA_ARCH__)
  return __umulhi(a, b);
#else
  return (uint32_t)(((uint64_t)a * (uint64_t)b) >> 32);
#endif
}

// Philox4x32 with 10 rounds; constants are those of the published generator.
PIMC_HD Philox4 philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                              uint32_t k0, uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
  const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
  for (int r = 0; r < 10; ++r) {
    const uint32_t lo0 = M0 * c0, hi0 = mulhi32(M0, c0);
    const uint32_t lo1 = M1 * c2, hi1 = mulhi32(M1, c2);
    const uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
    c0 = n0;
    c1 = lo1;
    c2 = n2;
    c3 = lo0;
    k0 += W0;
    k1 += W1;
  }
  Philox4 out;
  out.v[0] = c0;
  out.v[1] = c1;
  out.v[2] = c2;
  out.v[3] = c3;
  return out;
}

// 53 random bits -> uniform double in [0, 1); exact.
PIMC_HD double u53(uint32_t hi, uint32_t lo) {
  const uint64_t x = (((uint64_t)hi << 32) | (uint64_t)lo) >> 11;
  return (double)x * 1.1102230246251565404e-16;  // 2^-53
}

enum : uint32_t { kStreamUniform = 0u, kStreamNormal = 1u };

PIMC_HD double stream_uniform(uint64_t seed, uint32_t replica, uint32_t attempt,
                              uint32_t j) {
  const Philox4 b = philox4x32_10(j >> 1, attempt, replica, kStreamUniform,
                                  (uint32_t)seed, (uint32_t)(seed >> 32));
  return (j & 1u) ? u53(b.v[2], b.v[3]) : u53(b.v[0], b.v[1]);
}

// log(v) for v in [2^-53, 1]: exact split v = m 2^e with m in [sqrt(1/2), sqrt(2)),
// then 2 atanh(s), s = (m-1)/(m+1), |s| <= 0.1716, 11 odd terms.
PIMC_HD double portable_log(double v) {
  union {
    double d;
    uint64_t u;
  } c;
  c.d = v;
  int e = (int)((c.u >> 52) & 0x7ff) - 1023;
  c.u = (c.u & 0x000fffffffffffffull) | 0x3ff0000000000000ull;  // m in [1,2)
  double m = c.d;
  if (m > 1.4142135623730951) {
    m = PR_MUL(m, 0.5);
    e += 1;
  }
  const double s = PR_DIV(PR_SUB(m, 1.0), PR_ADD(m, 1.0));
  const double s2 = PR_MUL(s, s);
  double p = (1.0 / 23.0);
  p = PR_FMA(p, s2, (1.0 / 21.0));
  p = PR_FMA(p, s2, (1.0 / 19.0));
  p = PR_FMA(p, s2, (1.0 / 17.0));
  p = PR_FMA(p, s2, (1.0 / 15.0));
  p = PR_FMA(p, s2, (1.0 / 13.0));
  p = PR_FMA(p, s2, (1.0 / 11.0));
  p = PR_FMA(p, s2, (1.0 / 9.0));
  p = PR_FMA(p, s2, (1.0 / 7.0));
  p = PR_FMA(p, s2, (1.0 / 5.0));
  p = PR_FMA(p, s2, (1.0 / 3.0));
  const double t = PR_MUL(2.0, s);                       // exact
  const double logm = PR_FMA(PR_MUL(t, s2), p, t);        // 2s + 2s^3 p(s^2)
  const double LN2_HI = 6.93147180369123816490e-01;       // ln 2, high 32 bits
  const double LN2_LO = 1.90821492927058770002e-10;       // ln 2 - LN2_HI
  const double de = (double)e;
  return PR_ADD(PR_MUL(de, LN2_HI), PR_FMA(de, LN2_LO, logm));
}

// cos(2 pi u), sin(2 pi u) for u in [0,1): quarter-turn reduction is exact
// because u is a multiple of 2^-53; |x| <= pi/4 after it.
PIMC_HD void portable_cossin_2pi(double u, double* cs, double* sn) {
  const double t = PR_MUL(u, 4.0);  // exact
  double q = (double)(int)(PR_ADD(t, 0.5));
  const double f = PR_SUB(t, q);    // exact, in [-0.5, 0.5]
  const double HALF_PI = 1.57079632679489661923;
  const double x = PR_MUL(f, HALF_PI);
  const double x2 = PR_MUL(x, x);
  // sin x = x (1 - x^2/3! + x^4/5! - ... - x^20/21!)
  double ps = -(1.0 / 51090942171709440000.0);          // -1/21!
  ps = PR_FMA(ps, x2, (1.0 / 121645100408832000.0));    // 1/19!
  ps = PR_FMA(ps, x2, -(1.0 / 355687428096000.0));      // -1/17!
  ps = PR_FMA(ps, x2, (1.0 / 1307674368000.0));         // 1/15!
  ps = PR_FMA(ps, x2, -(1.0 / 6227020800.0));           // -1/13!
  ps = PR_FMA(ps, x2, (1.0 / 39916800.0));              // 1/11!
  ps = PR_FMA(ps, x2, -(1.0 / 362880.0));               // -1/9!
  ps = PR_FMA(ps, x2, (1.0 / 5040.0));                  // 1/7!
  ps = PR_FMA(ps, x2, -(1.0 / 120.0));                  // -1/5!
  ps = PR_FMA(ps, x2, (1.0 / 6.0));                     // 1/3!
  const double s = PR_FMA(PR_MUL(-x, x2), ps, x);
  // cos x = 1 - x^2/2! + x^4/4! - ... + x^22/22!
  double pc = -(1.0 / 1124000727777607680000.0);        // -1/22!
  pc = PR_FMA(pc, x2, (1.0 / 2432902008176640000.0));   // 1/20!
  pc = PR_FMA(pc, x2, -(1.0 / 6402373705728000.0));     // -1/18!
  pc = PR_FMA(pc, x2, (1.0 / 20922789888000.0));        // 1/16!
  pc = PR_FMA(pc, x2, -(1.0 / 87178291200.0));          // -1/14!
  pc = PR_FMA(pc, x2, (1.0 / 479001600.0));             // 1/12!
  pc = PR_FMA(pc, x2, -(1.0 / 3628800.0));              // -1/10!
  pc = PR_FMA(pc, x2, (1.0 / 40320.0));                 // 1/8!
  pc = PR_FMA(pc, x2, -(1.0 / 720.0));                  // -1/6!
  pc = PR_FMA(pc, x2, (1.0 / 24.0));                    // 1/4!
  pc = PR_FMA(pc, x2, -0.5);
  const double c = PR_FMA(x2, pc, 1.0);
  const int iq = ((int)q) & 3;
  if (iq == 0) {
    *cs = c;
    *sn = s;
  } else if (iq == 1) {
    *cs = -s;
    *sn = c;
  } else if (iq == 2) {
    *cs = -c;
    *sn = -s;
  } else {
    *cs = s;
    *sn = -c;
  }
}

// Normal pair from one Philox block (Box-Muller with radius sqrt(-2 log(1-u1))).
PIMC_HD void stream_normal_pair(uint64_t seed, uint32_t replica, uint32_t attempt,
                                uint32_t pair, double* z0, double* z1) {
  const Philox4 b = philox4x32_10(pair, attempt, replica, kStreamNormal,
                                  (uint32_t)seed, (uint32_t)(seed >> 32));
  const double u1 = u53(b.v[0], b.v[1]);
  const double u2 = u53(b.v[2], b.v[3]);
  const double rad = PR_SQRT(PR_MUL(-2.0, portable_log(PR_SUB(1.0, u1))));
  double c, s;
  portable_cossin_2pi(u2, &c, &s);
  *z0 = PR_MUL(rad, c);
  *z1 = PR_MUL(rad, s);
}

PIMC_HD double stream_normal(uint64_t seed, uint32_t replica, uint32_t attempt,
                             uint32_t k) {
  double z0, z1;
  stream_normal_pair(seed, replica, attempt, k >> 1, &z0, &z1);
  return (k & 1u) ? z1 : z0;
}

}  // namespace pimc
