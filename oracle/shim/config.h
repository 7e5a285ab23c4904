/* Build configuration for compiling pi-qmc's hot-path sources as the test oracle
   (stands in for the autotools-generated config.h; serial, 3-D, no MPI/SPRNG). */
#ifndef PIMC_ORACLE_CONFIG_H
#define PIMC_ORACLE_CONFIG_H
#define NDIM 3
#define HAVE_CONFIG_H 1
/* LAPACK comes from scipy's bundled OpenBLAS, whose symbols carry a scipy_ prefix. */
#define F77_FUNC(name, NAME) scipy_##name##_
#endif
