// Runs pi-qmc's own samplers on the pi-qmc-side adapters (GpuAdapters.cc) and
// writes what they produced, for tests/test_adapters.py to hold against the
// golden records pi-qmc made without them.  TEST INFRASTRUCTURE: linked
// against oracle/_ref/libpimcref.so (pi-qmc's objects and the replay driver)
// and tests/adapters/standin_engine.cc (the C ABI computed by oracle/port.cc).
//
//   adapter_check <input> <output>
// input:  ora_config, int ntab, per table {int s1, s2, ngpts, norder;
//         double rgridinv, logrratioinv; ugrid}, [has_ewald, totk, kvec, vk,
//         one_over_2v, self_energy, ikmax[3]], the initial path, int nattempt
// output: ora_record[nattempt] from MultiLevelSampler / DoubleMLSampler with
//         GpuCompositeAction in place of the composite action and GpuNodeModel
//         in place of each species' node model; then the path after
//         GpuSectionSampler ran nattempt attempts on pi-qmc's Paths, the
//         gpuThermoEnergy of that path, and three stand-in call counts.
#include <cstdio>
#include <cstdlib>
#include <stdexcept>
#include <vector>

#include "GpuAdapters.h"
#include "base/Paths.h"
#include "base/SimulationInfo.h"
#include "oracle_api.h"

extern "C" {
void* ref_create(const ora_config* c);
void ref_set_path(void* h, const double* xyz);
void ref_get_path(void* h, double* xyz);
int ref_run(void* h, int n, uint32_t first_attempt, ora_record* recs);
void ref_replace_action(void* h, void* action);
int ref_replace_node_model(void* h, int ispec, void* model);
void* ref_paths(void* h);
void* ref_simulation_info(void* h);
void standin_counts(pimc_engine* e, int* node, int* action, int* pushes);
}

namespace {
FILE* in = 0;
template <class T>
void get(T* p, size_t n) {
  if (fread(p, sizeof(T), n, in) != n) throw std::runtime_error("short input");
}

pimc_engine* make_engine(void* h, const ora_config& c, std::vector<pimc_pair_table>& tabs,
                         const pimc_ewald_table* ew) {
  pimc_gb300::SystemOptions opt;
  opt.nlevel = c.nlevel;
  opt.spring = c.spring != 0;
  opt.coulomb = c.coulomb != 0;
  opt.ewald = c.ewald != 0;
  opt.pbc_mover = c.mover == 1;
  opt.epsilon = c.epsilon;
  for (int i = 0; i < c.nspecies; ++i) {
    opt.sho_omega.push_back(c.sho_omega[i]);
    opt.node_kind.push_back(c.node_kind[i]);
    opt.node_omega.push_back(c.node_omega[i]);
  }
  opt.node_temperature = c.node_temperature;
  pimc_system sys =
      pimc_gb300::systemFromSimulation(*(const SimulationInfo*)ref_simulation_info(h), opt);
  for (int i = 0; i < c.nspecies; ++i) {
    sys.prim_a[i] = c.prim_a[i];
    sys.prim_b[i] = c.prim_b[i];
  }
  pimc_engine* e = 0;
  pimc_gb300::check(pimc_engine_create(&sys, 1, tabs.empty() ? 0 : &tabs[0], (int)tabs.size(),
                                       ew, c.seed, PIMC_PREC_FP64, &e),
                    "pimc_engine_create");
  return e;
}
}  // namespace

int main(int argc, char** argv) {
  if (argc != 3) return 2;
  in = fopen(argv[1], "rb");
  if (!in) return 2;
  ora_config c;
  get(&c, 1);
  int ntab = 0;
  get(&ntab, 1);
  std::vector<pimc_pair_table> tabs(ntab);
  std::vector<std::vector<double> > grids(ntab);
  for (int k = 0; k < ntab; ++k) {
    int hd[4];
    double gp[2];
    get(hd, 4);
    get(gp, 2);
    grids[k].resize((size_t)hd[2] * 2 * (hd[3] + 1));
    get(&grids[k][0], grids[k].size());
    pimc_pair_table& t = tabs[k];
    t.species1 = hd[0];
    t.species2 = hd[1];
    t.ngpts = hd[2];
    t.norder = hd[3];
    t.rgridinv = gp[0];
    t.logrratioinv = gp[1];
    t.ugrid = &grids[k][0];
  }
  int has_ew = 0;
  get(&has_ew, 1);
  pimc_ewald_table ew;
  std::vector<int> kvec;
  std::vector<double> vk;
  if (has_ew) {
    get(&ew.totk, 1);
    kvec.resize(3 * ew.totk);
    vk.resize(ew.totk);
    get(&kvec[0], kvec.size());
    get(&vk[0], vk.size());
    get(&ew.one_over_2v, 1);
    get(&ew.self_energy, 1);
    get(ew.ikmax, 3);
    ew.kvec = &kvec[0];
    ew.vk = &vk[0];
  }
  std::vector<double> path0((size_t)c.nslice * c.npart * 3);
  get(&path0[0], path0.size());
  int n = 0;
  get(&n, 1);
  fclose(in);

  // (1) pi-qmc's samplers and FixedNodeAction on GpuCompositeAction / GpuNodeModel
  void* h = ref_create(&c);
  pimc_engine* e = make_engine(h, c, tabs, has_ew ? &ew : 0);
  ref_replace_action(h, new pimc_gb300::GpuCompositeAction(e, c.npart, c.nlevel));
  for (int sp = 0; sp < c.nspecies; ++sp)
    if (c.node_kind[sp] &&
        ref_replace_node_model(h, sp, (NodeModel*)new pimc_gb300::GpuNodeModel(
                                          e, sp, c.npart, c.spec_count[sp], c.nlevel)) != 0)
      return 3;
  ref_set_path(h, &path0[0]);
  std::vector<ora_record> recs(n);
  ref_run(h, n, 0, &recs[0]);
  int counts[3];
  standin_counts(e, &counts[0], &counts[1], &counts[2]);

  // (2) GpuSectionSampler and gpuThermoEnergy on pi-qmc's Paths
  void* h2 = ref_create(&c);
  Paths& paths = *(Paths*)ref_paths(h2);
  ref_set_path(h2, &path0[0]);
  pimc_engine* e2 = make_engine(h2, c, tabs, has_ew ? &ew : 0);
  pimc_gb300::GpuSectionSampler sampler(paths, e2, n);
  sampler.run();
  std::vector<double> path1(path0.size());
  ref_get_path(h2, &path1[0]);
  const double energy = pimc_gb300::gpuThermoEnergy(paths, e2);

  FILE* out = fopen(argv[2], "wb");
  if (!out) return 2;
  fwrite(&recs[0], sizeof(ora_record), n, out);
  fwrite(&path1[0], sizeof(double), path1.size(), out);
  fwrite(&energy, sizeof(double), 1, out);
  fwrite(counts, sizeof(int), 3, out);
  fclose(out);
  return 0;
}
