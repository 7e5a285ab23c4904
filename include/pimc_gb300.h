/* pimc_gb300 — C ABI of the GB300 (sm_103a) path-integral Monte Carlo engine.
 *
 * The engine runs pi-qmc's multilevel-bisection hot path on the GPU: the
 * action difference of a bisection move (kinetic spring, harmonic and
 * primitive confinement, tabulated Coulomb pair action with Ewald long-range
 * term), the fixed-node Slater-determinant check on every changed slice with
 * the nodal action, the free-particle bisection mover, the section choosers,
 * and the thermodynamic energy estimator.  Each entry point below names the
 * pi-qmc interface it replaces (file:line in the reference tree).
 *
 * Conventions
 *  - Every function returns PIMC_OK (0) or a negative PIMC_ERR_* code; the
 *    message of the last failure is available from pimc_last_error().  Nothing
 *    here calls exit(): pi-qmc's exit-on-error paths
 *    (src/fixednode/SHONodes.cc:86-111, src/fixednode/FixedNodeAction.cc:342-349)
 *    become per-replica status words (pimc_replica_status).
 *  - Host arrays are caller-owned and plain C; device memory is owned by the
 *    engine.  Paths are [replica][slice][particle][xyz] doubles, i.e. pi-qmc's
 *    Beads storage (src/base/Beads.h:131-225) with slices outermost.
 *  - Work is issued on the stream set by pimc_set_stream (default: the legacy
 *    default stream); calls that return host data synchronize that stream.
 */
#ifndef PIMC_GB300_H
#define PIMC_GB300_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PIMC_MAX_SPECIES 4
#define PIMC_MAX_LEVEL 6
#define PIMC_MAX_NODE_PARTICLES 32

enum {
  PIMC_OK = 0,
  PIMC_ERR_INVALID = -1,     /* bad argument or unsupported configuration */
  PIMC_ERR_CUDA = -2,        /* a CUDA runtime call failed */
  PIMC_ERR_NO_DEVICE = -3,   /* no sm_103a device */
  PIMC_ERR_CAPACITY = -4     /* a size beyond a documented maximum */
};

/* Node models (src/fixednode/SHONodes.h, src/fixednode/FreeParticleNodes.h). */
enum { PIMC_NODES_NONE = 0, PIMC_NODES_SHO = 1, PIMC_NODES_FREE = 2 };
/* Bisection movers (src/advancer/mover/FreeMover.h, FreeMoverPBC.h). */
enum { PIMC_MOVER_FREE = 0, PIMC_MOVER_FREE_PBC = 1 };
/* Arithmetic of the move kernels. */
enum {
  PIMC_PREC_FP64 = 0,  /* everything in FP64: the plain form, parity with pi-qmc */
  PIMC_PREC_MIXED = 1  /* FP32 spring/pair sums with compensated accumulation;
                          FP64 determinants, sign tests, Ewald phases, totals */
};

/* One simulated system: what pi-qmc's SimulationInfo (src/base/SimulationInfo.h)
 * plus the action/sampler XML attributes describe.  Species occupy consecutive
 * particle ranges in order. */
typedef struct {
  int npart;
  int nspecies;
  int spec_count[PIMC_MAX_SPECIES];
  double spec_mass[PIMC_MAX_SPECIES];
  double spec_charge[PIMC_MAX_SPECIES];
  double sho_omega[PIMC_MAX_SPECIES];  /* >0: SHOAction on the species */
  double prim_a[PIMC_MAX_SPECIES];     /* PrimSHOAction a x^2 + b x^4 */
  double prim_b[PIMC_MAX_SPECIES];
  int node_kind[PIMC_MAX_SPECIES];     /* PIMC_NODES_* per species */
  double node_omega[PIMC_MAX_SPECIES];
  double node_temperature;             /* trial density-matrix temperature */
  int nslice;
  double tau;
  int nlevel;                          /* sections hold 2^nlevel + 1 slices */
  double cell[3];
  int spring;                          /* SpringAction on */
  int coulomb;                         /* CoulombAction on (needs pair tables) */
  double epsilon;
  int ewald;                           /* long-range Ewald term (needs an Ewald table) */
  int mover;                           /* PIMC_MOVER_* */
  /* Sampler attributes of pi-qmc's <Sample> (src/parser/PIMCParser.cc:312-322),
   * read by MultiLevelSampler / DoubleMLSampler.  Zero-initialised they are
   * pi-qmc's defaults.  Every level's bisection width is
   * sigma_factor sqrt(lambda tau 2^l) (defaultSigmaFactor; 0 means 1).  With
   * delayed_rejection != 0, a level-(nlevel - 1) move that its uniform rejects
   * gets a second proposal of width dr_sigma_factor sqrt(lambda tau 2^l)
   * (newSigmaFactor; 0 means 0.75) and the delayed-rejection acceptance of
   * src/advancer/MultiLevelSampler.cc:114-148 and
   * src/advancer/DoubleMLSampler.cc:148-204.  Delayed rejection needs
   * PIMC_MOVER_FREE (FreeMoverPBC leaves the forward probability of its first
   * proposal unset). */
  int delayed_rejection;
  double sigma_factor;
  double dr_sigma_factor;
} pimc_system;

/* A tabulated pair action, pi-qmc's PairAction::ugrid(ngpts,2,norder+1) on a
 * logarithmic grid (src/action/PairAction.cc:161-185,601-655), row-major
 * (index (i*2+t)*(norder+1)+k; t=0 action, t=1 tau derivative). */
typedef struct {
  int species1, species2;
  int ngpts, norder;
  double rgridinv, logrratioinv;
  const double* ugrid;
} pimc_pair_table;

/* Long-range Ewald data of an EwaldSum (src/util/EwaldSum.h:60-134): half-space
 * k-vectors (integer multiples of 2pi/L), their v_k, 1/(2V), self energy. */
typedef struct {
  int totk;
  const int* kvec; /* totk x 3 */
  const double* vk;
  double one_over_2v;
  double self_energy;
  int ikmax[3];
} pimc_ewald_table;

/* One attempted section move (for parity checks and statistics). */
typedef struct {
  int ifirst1, ifirst2;  /* section starts; ifirst2 = -2 without fixed node */
  int ipart;             /* moving particle */
  int reject_level;      /* level that rejected, -1 when accepted */
  double ds[PIMC_MAX_LEVEL + 3];       /* Action difference per level */
  double ds_node[PIMC_MAX_LEVEL + 3];  /* DoubleAction difference per level */
  double lnt[PIMC_MAX_LEVEL + 3];      /* mover ln(T_old/T_new) per level */
} pimc_move_record;

/* Per-replica status word bits. */
enum {
  PIMC_STATUS_INIT_CROSSING = 1,  /* node crossing found when a section was set up */
  PIMC_STATUS_SINGULAR = 2,       /* a Slater matrix had an exactly zero pivot */
  PIMC_STATUS_RESCALE_LIMIT = 4,  /* determinant rescaling hit its iteration limit */
  PIMC_STATUS_NONFINITE = 8       /* a non-finite bead coordinate arrived (pimc_upload_paths,
                                     pimc_server_admit) or a move's action or ln T was not finite */
};

typedef struct pimc_engine pimc_engine;

/* ---- lifetime ---------------------------------------------------------- */

/* Creates an engine holding nreplica copies of one system, each with its own
 * path and random stream (replica r draws stream r of the seed).  Replaces the
 * object graph pi-qmc's parsers build for one clone
 * (src/parser/ActionParser.cc:105-153,433-452, src/parser/PIMCParser.cc:312-491):
 * SpringAction, SHOAction, PrimSHOAction, CoulombAction (from the given pair
 * tables and Ewald table), FixedNodeAction with SHONodes/FreeParticleNodes,
 * FreeMover/FreeMoverPBC, SectionChooser or DoubleSectionChooser, and a
 * MultiLevelSampler/DoubleMLSampler moving one particle chosen by
 * SimpleParticleChooser. */
int pimc_engine_create(const pimc_system* sys, int nreplica, const pimc_pair_table* tables,
                       int ntables, const pimc_ewald_table* ewald, uint64_t seed,
                       int precision, pimc_engine** out);

/* Creates an engine whose replicas are different systems (uneven particle
 * counts, slice counts, levels, frequencies): the batched form.  sys[r] is
 * replica r's system; table_offset[r]..table_offset[r+1] index its pair tables. */
int pimc_engine_create_batch(const pimc_system* sys, int nreplica,
                             const pimc_pair_table* tables, const int* table_offset,
                             uint64_t seed, int precision, pimc_engine** out);

int pimc_engine_destroy(pimc_engine* e);
const char* pimc_last_error(void);
/* cudaStream_t to issue work on (NULL: legacy default stream). */
int pimc_set_stream(pimc_engine* e, void* stream);

/* ---- paths (SerialPaths::getBeads/putBeads, src/base/SerialPaths.cc:119-185) */

/* Host <-> device copies of all replicas' paths (host layout above).  An
 * upload rebuilds the cached per-slice results (Slater entries, structure
 * factors) of the slices whose beads changed, bit for bit as a full rebuild. */
int pimc_upload_paths(pimc_engine* e, const double* host_xyz);
int pimc_download_paths(pimc_engine* e, double* host_xyz);
/* Offsets (in doubles) of each replica's path in the packed host layout; for
 * engines of one system this is r * nslice * npart * 3. */
int pimc_path_offsets(pimc_engine* e, int64_t* offsets /* nreplica+1 */);

/* ---- checkpoints (WritePaths / PathReader, and the random-stream position) */

/* Path files in pi-qmc's restart format: "#Permutations ..." (the identity),
 * "#Path coordinates: N particles in 3-d", then one line per slice with every
 * particle's x y z at 15 significant digits, each followed by a space
 * (WritePaths::run, src/algorithm/WritePaths.cc:25-114).  xyz is one
 * replica's host path, [nslice][npart][3]. */
int pimc_paths_write_file(const char* filename, const double* xyz, int npart, int nslice);
/* Reads such a file as PathReader::run does (src/algorithm/PathReader.cc:20-140):
 * the "#Permutations" line is optional (without it a last, wrapped slice is
 * read and matched to the first), file slice k fills slices
 * k + ib*nslice/bfactor for ib < bfactor.  Files whose permutation is not the
 * identity, that end early or that hold a non-number are rejected
 * (PIMC_ERR_INVALID); xyz is left unchanged then. */
int pimc_paths_read_file(const char* filename, double* xyz, int npart, int nslice, int bfactor);
/* The same for replica `replica` of an engine (an active slot of a server for
 * writing).  Reading replaces that replica's path only and rebuilds its cached
 * Slater results; servers take paths at admission instead. */
int pimc_write_paths(pimc_engine* e, int replica, const char* filename);
int pimc_read_paths(pimc_engine* e, int replica, const char* filename, int bfactor);

/* Everything besides the path that decides a replica's future moves: the
 * position of its random stream (attempts made), its acceptance counts and
 * status word, and the node models' determinant scales (SHONodes /
 * FreeParticleNodes rescale the matrix to keep det in range).  A replica whose
 * path (exact doubles: pimc_download_paths / pimc_upload_paths) and state are
 * copied into another engine of the same system and seed continues the
 * identical chain. */
typedef struct {
  uint32_t attempt;   /* section/displace attempts drawn from the replica's stream */
  uint32_t status;    /* PIMC_STATUS_* bits */
  int64_t accepted, attempted;
  double node_scale[PIMC_MAX_SPECIES];
} pimc_replica_state;
int pimc_get_replica_state(pimc_engine* e, int replica, pimc_replica_state* out);
int pimc_set_replica_state(pimc_engine* e, int replica, const pimc_replica_state* in);

/* ---- the sampler ------------------------------------------------------- */

/* Runs nattempt section-move attempts on every replica, on the device, in
 * pi-qmc's order: SectionChooser::run (src/advancer/SectionChooser.cc:30-48) or
 * DoubleSectionChooser::run (src/advancer/DoubleSectionChooser.cc:33-65) around
 * MultiLevelSampler::tryMove (src/advancer/MultiLevelSampler.cc:100-177) or
 * DoubleMLSampler::tryMove (src/advancer/DoubleMLSampler.cc:123-245).
 * Asynchronous on the engine's stream.  records (optional, host) receives
 * nreplica*nattempt records, replica-major; requesting them synchronizes. */
int pimc_run_sections(pimc_engine* e, int nattempt, pimc_move_record* records);

/* Per-replica accepted-move counts and status words since creation. */
int pimc_replica_status(pimc_engine* e, int64_t* accepted, int64_t* attempted,
                        uint32_t* status);

/* Runs nsteps steps, each nattempt section attempts on every replica followed by
 * one energy measurement of every replica, as one CUDA graph (captured on the
 * first call with these arguments, replayed afterwards).  host_energy, when not
 * NULL, receives [nsteps][nreplica] energies and the call waits for them;
 * otherwise it returns once the graph is enqueued.  This is pi-qmc's
 * <Loop><ChooseSection/><Sample/><Measure/></Loop> body (src/parser/PIMCParser.cc)
 * with the ThermoEnergyEstimator as the measurement. */
int pimc_run_steps(pimc_engine* e, int nattempt, int nsteps, double* host_energy);

/* ---- rigid displacement moves ------------------------------------------- */

/* One attempted rigid displacement of whole particle paths. */
typedef struct {
  int ipart[4];       /* moving particles (-1 past nmoving) */
  double disp[4][3];  /* their displacements */
  double ds;          /* Action difference (both halves of the path for fixed node) */
  double ds_node;     /* fixed-node (DoubleAction) difference */
  int accepted;
} pimc_displace_record;

/* nattempt rigid-displacement attempts on every replica: DisplaceMoveSampler
 * (src/advancer/DisplaceMoveSampler.cc:63-224), or DoubleDisplaceMoveSampler
 * (src/advancer/DoubleDisplaceMoveSampler.cc:40-128) for fixed-node systems, with
 * a UniformMover of box box[3] (src/advancer/UniformMover.cc:25-42), nmoving
 * (1..4) particles chosen from all particles (species < 0) or from one
 * species.  records: [nreplica][nattempt] or NULL. */
int pimc_run_displace(pimc_engine* e, int nattempt, const double* box, int nmoving, int species,
                      pimc_displace_record* records);

/* ---- further estimators ------------------------------------------------- */

/* Virial energy estimator with window nwindow (VirialEnergyEstimator,
 * src/estimator/VirialEnergyEstimator.cc:34-79) of every replica, FP64.
 * nwindow = 1 gives the thermodynamic estimator's value. */
int pimc_virial_energy(pimc_engine* e, int nwindow, double* host_energy /* nreplica */);
/* Coulomb potential energy, direct pair sum with minimum image
 * (CoulombEnergyEstimator, src/estimator/CoulombEnergyEstimator.cc:30-44). */
int pimc_coulomb_energy(pimc_engine* e, double epsilon, double* host_energy);
/* Coulomb potential energy with the estimator's own optimized Ewald sum
 * (EwaldCoulombEstimator, src/estimator/EwaldCoulombEstimator.cc:60-140): est and
 * vgrid (1001 doubles) from pimc_ewald_estimator_tables. */
int pimc_ewald_coulomb_energy(pimc_engine* e, double epsilon, double rcut,
                              const pimc_ewald_table* est, const double* vgrid,
                              double* host_energy);
/* Builds that Ewald table and grid for a system (host only, no GPU). */
int pimc_ewald_estimator_tables(const pimc_system* sys, double rcut, double kcut, double epsilon,
                                const pimc_ewald_table** est, double* vgrid);

/* ---- host-built action tables (no GPU) ----------------------------------- */

/* The tables CoulombAction's constructor builds (src/action/CoulombAction.cc:19-91
 * with PairAction's empirical-action grid, src/action/PairAction.cc:161-185):
 * one pair table per interacting species pair i <= j, and with sys->ewald the
 * OptEwaldSum long-range table (src/util/OptEwaldSum.cc:28-245) for real-space
 * cutoff ewald_rcut (0: half the first box side) and k cutoff ewald_kcut.
 * ngpts 0 / rmin 0 / rmax 0 take pi-qmc's defaults.  The arrays stay valid
 * until the next call on the same thread; *ewald is NULL without Ewald. */
int pimc_coulomb_tables(const pimc_system* sys, int norder, int ngpts, double rmin, double rmax,
                        double ewald_rcut, double ewald_kcut, const pimc_pair_table** tables,
                        int* ntables, const pimc_ewald_table** ewald);
/* The short-range polynomial coefficients (n of them) of the last Ewald table
 * pimc_coulomb_tables built on this thread. */
int pimc_ewald_coefficients(double* coef, int n);

/* ---- launch configuration and autotuning -------------------------------- */

/* Launch configuration of an engine's section kernel: threads per replica
 * (64, 128, 256, or 512 with variant 1), where the per-warp Slater scratch lives (0: shared
 * memory where it fits; 1: global memory; 2: its hot part, the LU and inverse, in shared
 * memory and its cold part, the element and gradient matrices, in global memory, which
 * frees shared memory for more resident replicas), the replicas resident per SM (0: as
 * many as fit) and the section
 * kernel's register-budget variant.  ms is the
 * time the autotuner measured for it (0 when not measured).  A configuration
 * changes how per-thread partial sums are grouped, so chains run under two
 * configurations agree to rounding, not bit for bit. */
typedef struct {
  int block;
  int scratch_global;
  int ctas_per_sm;
  int regs_variant;  /* register budget: 65536 / (256 * regs_variant) per thread (2, 3 or 4;
                        0 = 2), or 1: the variant for up to 512 threads (128 registers) */
  float ms;
} pimc_launch_config;

/* On a server the configuration (block, scratch placement, register variant)
 * applies to every round and may be set only before the first admission, so
 * that a simulation's sums never depend on the mix it is served in. */
int pimc_engine_configure(pimc_engine* e, const pimc_launch_config* cfg);
int pimc_engine_get_config(pimc_engine* e, pimc_launch_config* cfg);
/* Times each candidate configuration on nattempt section attempts per replica
 * (paths, Slater caches and counters are restored after every trial, so tuning
 * does not advance the chains), applies the fastest and returns it in *best;
 * tried (up to max_tried entries, may be NULL) receives every candidate with
 * its time and *ntried their number. */
int pimc_engine_autotune(pimc_engine* e, int nattempt, pimc_launch_config* best,
                         pimc_launch_config* tried, int max_tried, int* ntried);

/* ---- serving ----------------------------------------------------------- */

/* A server runs many independent simulations that come and go: each admitted
 * simulation occupies a slot, its path and Slater-result cache live in one
 * device pool of hbm_bytes, and every pimc_server_run advances all admitted
 * slots in one persistent launch (continuous batching).  A simulation draws
 * the random stream of its own stream_id, so its chain is the same whether it
 * runs alone or among others.  The maxima fix the shared-memory layout. */
typedef struct {
  int slots;             /* concurrent simulations */
  size_t hbm_bytes;      /* device pool for paths and caches */
  int max_npart;
  int max_nslice;
  int max_level;
  int max_node_count;    /* largest node-model species (0: no node models) */
} pimc_server_config;

int pimc_server_create(const pimc_server_config* cfg, uint64_t seed, int precision,
                       pimc_engine** out);
/* Admits one simulation (system, its pair tables, its initial path
 * [nslice][npart][3]) that advances round_attempts section attempts in every
 * round; *slot receives its slot.  Returns PIMC_ERR_CAPACITY
 * when no slot is free or its path and cache do not fit the free pool (try
 * again after a release), PIMC_ERR_INVALID when the system exceeds the
 * server's maxima or needs Ewald sums. */
int pimc_server_admit(pimc_engine* e, const pimc_system* sys, const pimc_pair_table* tables,
                      int ntables, const double* host_path, uint32_t stream_id,
                      int round_attempts, int* slot);
int pimc_server_release(pimc_engine* e, int slot);
/* One round: every admitted slot advances its round_attempts section-move
 * attempts, all slots in one persistent launch (asynchronous). */
int pimc_server_run(pimc_engine* e);
/* Thermodynamic energy of every admitted slot (NaN for free slots). */
int pimc_server_energy(pimc_engine* e, double* energy /* slots */);
/* The same for the listed active slots only (energy[k] for slots[k]): a
 * serving loop measures a simulation once per sweep and at its end, not
 * every round.  A slot's value does not depend on which slots are listed. */
int pimc_server_energy_slots(pimc_engine* e, const int* slots, int nslot, double* energy);
int pimc_server_download_path(pimc_engine* e, int slot, double* host_xyz);
/* Bytes of the pool in use and free (largest free block). */
int pimc_server_pool(pimc_engine* e, size_t* used, size_t* largest_free);

/* ---- estimators -------------------------------------------------------- */

/* Thermodynamic energy estimator of every replica's current path:
 * (1/M) sum over links of utau, as ThermoEnergyEstimator::handleLink
 * (src/estimator/ThermoEnergyEstimator.cc:32-50) summing
 * CompositeAction::getBeadAction (src/action/CompositeAction.cc:59-69). */
int pimc_thermo_energy(pimc_engine* e, double* host_energy /* nreplica */);

/* ---- Action-level entry point ----------------------------------------- */

/* Action::getActionDifference(const SectionSamplerInterface&, int level)
 * (src/action/Action.h:44, src/action/CompositeAction.cc:30-37) for nbatch
 * independent sections of replica 0's system: section[b] is
 * [2^nlevel+1][npart][3], moving[b] is [2^nlevel+1][3] for particle ipart[b].
 * Returns the composite difference (spring + SHO + PrimSHO + Coulomb, Ewald at
 * level 0) per batch entry in ds[b]. Host arrays; synchronous. */
int pimc_action_difference(pimc_engine* e, int level, int nbatch, const double* section,
                           const double* moving, const int* ipart, double* ds);

/* ---- NodeModel-level entry point --------------------------------------- */

/* NodeModel::evaluate + evaluateDistance (src/fixednode/NodeModel.h:74-90,
 * src/fixednode/SHONodes.cc:51-170, src/fixednode/FreeParticleNodes.cc:72-234)
 * for species ispec of replica 0's system on nbatch slice pairs: r1[b], r2[b]
 * are [npart][3].  det[b] gets the Slater determinant (at the engine's current
 * scale for that species, no rescaling), d1[b]/d2[b] ([npart]) the nodal
 * distances (200 for particles of other species), err[b] 1 for a singular
 * matrix.  Host arrays; synchronous. */
int pimc_node_evaluate(pimc_engine* e, int ispec, int nbatch, const double* r1,
                       const double* r2, double* det, double* d1, double* d2, int* err);
int pimc_node_scale(pimc_engine* e, int replica, int ispec, double* scale);

/* ---- allocation-free NodeModel-level entry point ------------------------ */

/* The same node-model evaluation as pimc_node_evaluate, for callers that
 * cannot allocate GPU memory: host code that runs inside another framework's
 * memory budget or pool, or that must not call cudaMalloc/cudaFree on a
 * latency-critical path.  No engine is needed and nothing is allocated: sys is
 * read by value, r1/r2 ([nbatch][npart][3]) and det/err ([nbatch]),
 * d1/d2 ([nbatch][npart]) are the caller's DEVICE buffers, the Slater-matrix
 * scratch is a fixed 6.1 MiB static device array (128 slots of 6208 doubles),
 * and the kernel is issued on `stream` (cudaStream_t, NULL = legacy default).
 * scale is the node model's current scale (pimc_node_scale).  Limits: node
 * species of at most 32 particles, npart <= 1024; larger sizes return
 * PIMC_ERR_CAPACITY.  The first call on a device looks up the scratch array's
 * device address on that device, so make it before any stream capture; the
 * address is kept until exit, so a device reset (cudaDeviceReset) between calls
 * is not supported.  Every
 * call shares the one scratch array: calls that overlap on the GPU race and
 * must be ordered by the caller (one stream, or events).  Asynchronous.
 * This entry point has no counterpart in the reference. */
int pimc_node_evaluate_noalloc(const pimc_system* sys, int ispec, double scale, int nbatch,
                               const double* r1, const double* r2, double* det, double* d1,
                               double* d2, int* err, void* stream);

/* ---- random streams ---------------------------------------------------- */

/* The first n uniforms and n normals of replica `replica`'s attempt `attempt`
 * (the numbers the sampler consumes in place of pi-qmc's RandomNumGenerator,
 * src/util/RandomNumGenerator.h:41-85), generated on the device; lets a CPU
 * replay check it consumes bit-identical numbers.  Synchronous. */
int pimc_stream_sample(uint64_t seed, uint32_t replica, uint32_t attempt, int n,
                       double* uniforms, double* normals);

/* ---- timing ------------------------------------------------------------ */

/* Measured dense FP64 FMA throughput of the current device in TFLOP/s (a
 * short probe kernel; the roofline denominator for the FP64-bound kernels). */
int pimc_fp64_peak(double* tflops);
/* The same for FP32 FMAs (the denominator of the mixed form's FP32 work). */
int pimc_fp32_peak(double* tflops);

/* Kernel launches issued by this engine so far (for launch accounting). */
int64_t pimc_kernel_launches(pimc_engine* e);

#ifdef __cplusplus
}
#endif
#endif
