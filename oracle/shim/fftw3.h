/* Type-only stand-in for fftw3.h: PairIntegrator.h names these types, but no
   FFTW routine runs on the bisection path. */
#ifndef PIMC_ORACLE_FFTW3_H
#define PIMC_ORACLE_FFTW3_H
typedef double fftw_complex[2];
typedef struct fftw_plan_s* fftw_plan;
#endif
