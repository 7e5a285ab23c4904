// A stand-in for libpimc_gb300 behind the subset of include/pimc_gb300.h that
// the pi-qmc adapters (pi-qmc_gb300/adapters/GpuAdapters.cc) call, computed by
// the CPU restatement (oracle/port.cc) instead of the GPU.  TEST
// INFRASTRUCTURE: it lets the adapters run inside pi-qmc's own samplers on a
// machine without a GPU, so that the wiring (argument packing, per-slice
// node results, rescaling, path copies) is checked against pi-qmc's records.
// The engine's own parity with the restatement is held by the GPU tests.
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/pimc_gb300.h"
#include "../../oracle/oracle_api.h"

extern "C" {
void* port_create(const ora_config* c, int npair_tables, const int* pair_species,
                  const ora_pair_table* tables, const ora_ewald_table* ew);
void port_set_path(void* h, const double* xyz);
void port_get_path(void* h, double* xyz);
int port_run(void* h, int n, uint32_t first_attempt, ora_record* recs);
double port_thermo_energy(void* h);
double port_action_diff(void* h, int level, const double* section, const double* moving,
                        int ipart);
int port_node_eval(void* h, int ispec, const double* r1, const double* r2, int islice,
                   int scale_magnitude, double* det, double* d1, double* d2);
void port_set_node_scale(void* h, int ispec, double scale);
}

struct pimc_engine {
  void* port;
  pimc_system sys;
  pimc_replica_state state;
  int calls_node, calls_action, scale_pushes;
};

namespace {
std::string g_error;
int fail(int rc, const char* msg) {
  g_error = msg;
  return rc;
}
}  // namespace

extern "C" {

const char* pimc_last_error(void) { return g_error.c_str(); }

int pimc_engine_create(const pimc_system* sys, int nreplica, const pimc_pair_table* tables,
                       int ntables, const pimc_ewald_table* ewald, uint64_t seed, int precision,
                       pimc_engine** out) {
  if (!sys || nreplica != 1 || !out || precision != PIMC_PREC_FP64)
    return fail(PIMC_ERR_INVALID, "stand-in: one FP64 replica");
  ora_config c;
  memset(&c, 0, sizeof(c));
  c.npart = sys->npart;
  c.nspecies = sys->nspecies;
  for (int i = 0; i < sys->nspecies; ++i) {
    c.spec_count[i] = sys->spec_count[i];
    c.spec_mass[i] = sys->spec_mass[i];
    c.spec_charge[i] = sys->spec_charge[i];
    c.sho_omega[i] = sys->sho_omega[i];
    c.prim_a[i] = sys->prim_a[i];
    c.prim_b[i] = sys->prim_b[i];
    c.node_kind[i] = sys->node_kind[i];
    c.node_omega[i] = sys->node_omega[i];
  }
  c.node_temperature = sys->node_temperature;
  c.nslice = sys->nslice;
  c.tau = sys->tau;
  c.temperature = 1.0 / (sys->tau * sys->nslice);
  c.nlevel = sys->nlevel;
  for (int d = 0; d < 3; ++d) c.cell[d] = sys->cell[d];
  c.spring = sys->spring;
  c.coulomb = sys->coulomb;
  c.epsilon = sys->epsilon;
  c.norder = ntables > 0 ? tables[0].norder : 3;
  c.ewald = sys->ewald;
  c.mover = sys->mover;
  c.delayed_rejection = sys->delayed_rejection;
  c.sigma_factor = sys->sigma_factor;
  c.dr_sigma_factor = sys->dr_sigma_factor;
  c.seed = seed;
  c.replica = 0;
  std::vector<int> species(2 * (ntables > 0 ? ntables : 1));
  std::vector<ora_pair_table> t(ntables > 0 ? ntables : 1);
  for (int k = 0; k < ntables; ++k) {
    species[2 * k] = tables[k].species1;
    species[2 * k + 1] = tables[k].species2;
    t[k].ngpts = tables[k].ngpts;
    t[k].norder = tables[k].norder;
    t[k].rgridinv = tables[k].rgridinv;
    t[k].logrratioinv = tables[k].logrratioinv;
    t[k].ugrid = tables[k].ugrid;
  }
  ora_ewald_table ew;
  if (ewald) {
    ew.totk = ewald->totk;
    ew.kvec = ewald->kvec;
    ew.vk = ewald->vk;
    ew.one_over_2v = ewald->one_over_2v;
    ew.self_energy = ewald->self_energy;
    for (int d = 0; d < 3; ++d) ew.ikmax[d] = ewald->ikmax[d];
  }
  pimc_engine* e = new pimc_engine();
  e->port = port_create(&c, ntables, &species[0], &t[0], ewald ? &ew : 0);
  e->sys = *sys;
  memset(&e->state, 0, sizeof(e->state));
  for (int k = 0; k < PIMC_MAX_SPECIES; ++k) e->state.node_scale[k] = 1.0;
  *out = e;
  return PIMC_OK;
}

int pimc_get_replica_state(pimc_engine* e, int replica, pimc_replica_state* out) {
  if (!e || replica != 0 || !out) return fail(PIMC_ERR_INVALID, "bad argument");
  *out = e->state;
  return PIMC_OK;
}

int pimc_set_replica_state(pimc_engine* e, int replica, const pimc_replica_state* in) {
  if (!e || replica != 0 || !in) return fail(PIMC_ERR_INVALID, "bad argument");
  for (int k = 0; k < PIMC_MAX_SPECIES; ++k)
    if (!(in->node_scale[k] > 0) || !std::isfinite(in->node_scale[k]))
      return fail(PIMC_ERR_INVALID, "node scales must be positive and finite");
  e->state = *in;
  e->scale_pushes++;
  return PIMC_OK;
}

// NodeModel::evaluate + evaluateDistance at the replica's current scale, no
// rescaling (the engine's contract).
int pimc_node_evaluate(pimc_engine* e, int ispec, int nbatch, const double* r1, const double* r2,
                       double* det, double* d1, double* d2, int* err) {
  if (!e || ispec < 0 || ispec >= e->sys.nspecies || !e->sys.node_kind[ispec])
    return fail(PIMC_ERR_INVALID, "species has no node model");
  const int np = e->sys.npart;
  for (int b = 0; b < nbatch; ++b) {
    port_set_node_scale(e->port, ispec, e->state.node_scale[ispec]);
    err[b] = port_node_eval(e->port, ispec, r1 + (size_t)b * np * 3, r2 + (size_t)b * np * 3, 0,
                            0, det + b, d1 + (size_t)b * np, d2 + (size_t)b * np);
  }
  e->calls_node += nbatch;
  return PIMC_OK;
}

int pimc_action_difference(pimc_engine* e, int level, int nbatch, const double* section,
                           const double* moving, const int* ipart, double* ds) {
  if (!e) return fail(PIMC_ERR_INVALID, "bad argument");
  const int nsec = (1 << e->sys.nlevel) + 1, np = e->sys.npart;
  for (int b = 0; b < nbatch; ++b)
    ds[b] = port_action_diff(e->port, level, section + (size_t)b * nsec * np * 3,
                             moving + (size_t)b * nsec * 3, ipart[b]);
  e->calls_action += nbatch;
  return PIMC_OK;
}

int pimc_upload_paths(pimc_engine* e, const double* host_xyz) {
  if (!e || !host_xyz) return fail(PIMC_ERR_INVALID, "bad argument");
  port_set_path(e->port, host_xyz);
  return PIMC_OK;
}

int pimc_download_paths(pimc_engine* e, double* host_xyz) {
  if (!e || !host_xyz) return fail(PIMC_ERR_INVALID, "bad argument");
  port_get_path(e->port, host_xyz);
  return PIMC_OK;
}

int pimc_run_sections(pimc_engine* e, int nattempt, pimc_move_record* records) {
  if (!e || nattempt < 0 || records) return fail(PIMC_ERR_INVALID, "bad argument");
  e->state.accepted += port_run(e->port, nattempt, e->state.attempt, 0);
  e->state.attempt += nattempt;
  e->state.attempted += nattempt;
  return PIMC_OK;
}

int pimc_thermo_energy(pimc_engine* e, double* host_energy) {
  if (!e || !host_energy) return fail(PIMC_ERR_INVALID, "bad argument");
  *host_energy = port_thermo_energy(e->port);
  return PIMC_OK;
}

// Table building is the engine's own (host) code, not part of what the stand-in
// computes; the tests that link it build engines from pi-qmc's tables.
int pimc_coulomb_tables(const pimc_system*, int, int, double, double, double, double,
                        const pimc_pair_table**, int*, const pimc_ewald_table**) {
  return fail(PIMC_ERR_INVALID, "stand-in: no table builder");
}

// Counters for the test: node evaluations, action differences, scale changes.
void standin_counts(pimc_engine* e, int* node, int* action, int* pushes) {
  *node = e->calls_node;
  *action = e->calls_action;
  *pushes = e->scale_pushes;
}

}  // extern "C"
