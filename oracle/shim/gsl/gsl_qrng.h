/* Minimal stand-in for GSL's quasi-random generator header.  SectionChooser
   allocates a Sobol generator but never draws from it on the bisection path. */
#ifndef PIMC_ORACLE_GSL_QRNG_H
#define PIMC_ORACLE_GSL_QRNG_H
typedef struct gsl_qrng_type_s { int unused; } gsl_qrng_type;
typedef struct gsl_qrng_s { int unused; } gsl_qrng;
static const gsl_qrng_type* const gsl_qrng_sobol = 0;
static inline gsl_qrng* gsl_qrng_alloc(const gsl_qrng_type*, unsigned int) { return 0; }
static inline void gsl_qrng_free(gsl_qrng*) {}
static inline int gsl_qrng_get(const gsl_qrng*, double*) { return 0; }
#endif
