/* C interface shared by the two CPU checkers under oracle/:
 *   - oracle/_ref/libpimcref.so : pi-qmc's own hot-path sources (compiled from the
 *     reference tree by oracle/build_ref.py, only where that tree exists), and
 *   - oracle/liboracle_port.so  : the plain C++ restatement in oracle/port.cc.
 * Both are TEST INFRASTRUCTURE: only tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline leg load them, as checkers.  The product never does.
 *
 * Layouts: a path is [nslice][npart][3] doubles; a section is
 * [2^nlevel+1][npart][3]; moving beads are [2^nlevel+1][nmoving][3].
 * A pair-action table is pi-qmc's ugrid(ngpts,2,norder+1) in row-major order
 * (index (i*2+t)*(norder+1)+k), see src/action/PairAction.h. */
#ifndef PIMC_ORACLE_API_H
#define PIMC_ORACLE_API_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

#define ORA_MAX_SPECIES 4
#define ORA_MAX_LEVEL 8

typedef struct {
  int npart;
  int nspecies;
  int spec_count[ORA_MAX_SPECIES];
  double spec_mass[ORA_MAX_SPECIES];
  double spec_charge[ORA_MAX_SPECIES];
  double sho_omega[ORA_MAX_SPECIES]; /* > 0 : SHOAction on the species */
  double prim_a[ORA_MAX_SPECIES];    /* PrimSHOAction a x^2 + b x^4 when a or b != 0 */
  double prim_b[ORA_MAX_SPECIES];
  int node_kind[ORA_MAX_SPECIES];    /* 0 none, 1 SHONodes, 2 FreeParticleNodes */
  double node_omega[ORA_MAX_SPECIES];
  double node_temperature;           /* temperature of the trial density matrix */
  int nslice;
  double tau;
  double temperature;
  int nlevel;
  double cell[3];
  int spring;                        /* SpringAction */
  int coulomb;                       /* CoulombAction */
  double epsilon;
  int norder;
  int ngpts;                         /* 0 -> 500 */
  int ewald;                         /* optEwald long range */
  double ewald_rcut;                 /* 0 -> L/2 */
  double ewald_kcut;
  int mover;                         /* 0 FreeMover, 1 FreeMoverPBC */
  uint64_t seed;
  uint32_t replica;
  /* <Sample> attributes (src/parser/PIMCParser.cc:312-322); 0 = pi-qmc's defaults */
  int delayed_rejection;             /* delayedRejection */
  double sigma_factor;               /* defaultSigmaFactor (0 -> 1) */
  double dr_sigma_factor;            /* newSigmaFactor (0 -> 0.75 with delayed rejection) */
} ora_config;

/* One attempted section move. */
typedef struct {
  int ifirst1, ifirst2; /* section starts (ifirst2 = -2 for single sections) */
  int ipart;            /* moving particle */
  int reject_level;     /* level that rejected, or -1 when accepted */
  double ds[ORA_MAX_LEVEL + 1];      /* Action difference per level (level index) */
  double ds_node[ORA_MAX_LEVEL + 1]; /* DoubleAction difference per level */
  double lnt[ORA_MAX_LEVEL + 1];     /* mover ln(T_old/T_new) per level */
} ora_record;

/* One attempted rigid displacement of whole particle paths. */
#define ORA_MAX_MOVING 4
typedef struct {
  int ipart[ORA_MAX_MOVING];       /* moving particles (nmoving used) */
  double disp[ORA_MAX_MOVING][3];  /* their displacements */
  double ds;                       /* Action difference (both halves for the double form) */
  double ds_node;                  /* DoubleAction difference */
  int accepted;
} ora_drecord;

/* Pair-action table handed to the port (the reference builds its own). */
typedef struct {
  int ngpts, norder;
  double rgridinv, logrratioinv;
  const double* ugrid; /* (ngpts,2,norder+1) */
} ora_pair_table;

typedef struct {
  int totk;
  const int* kvec;     /* totk x 3 */
  const double* vk;    /* totk */
  double one_over_2v;
  double self_energy;
  int ikmax[3];
} ora_ewald_table;

#ifdef __cplusplus
}
#endif
#endif
