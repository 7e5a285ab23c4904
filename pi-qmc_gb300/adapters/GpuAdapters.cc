#include "GpuAdapters.h"

#include <cstring>
#include <stdexcept>
#include <string>

#include "advancer/SectionSamplerInterface.h"
#include "base/Beads.h"
#include "base/Paths.h"
#include "base/SimulationInfo.h"
#include "base/Species.h"
#include "util/SuperCell.h"

namespace pimc_gb300 {

void check(int status, const char* what) {
  if (status != PIMC_OK)
    throw std::runtime_error(std::string(what) + ": " + pimc_last_error());
}

GpuCompositeAction::GpuCompositeAction(pimc_engine* engine, int npart, int nlevel)
    : engine(engine), npart(npart), nsec((1 << nlevel) + 1),
      section(3 * nsec * npart), moving(3 * nsec) {}

double GpuCompositeAction::getActionDifference(const SectionSamplerInterface& sampler,
                                               int level) {
  const Beads<NDIM>& sec = sampler.getSectionBeads();
  const Beads<NDIM>& mov = sampler.getMovingBeads();
  const IArray& index = sampler.getMovingIndex();
  if (index.size() != 1) throw std::runtime_error("GpuCompositeAction moves one particle");
  for (int t = 0; t < nsec; ++t) {
    for (int i = 0; i < npart; ++i)
      for (int d = 0; d < 3; ++d) section[(t * npart + i) * 3 + d] = sec(i, t)[d];
    for (int d = 0; d < 3; ++d) moving[t * 3 + d] = mov(0, t)[d];
  }
  const int ipart = index(0);
  double ds = 0;
  check(pimc_action_difference(engine, level, 1, &section[0], &moving[0], &ipart, &ds),
        "pimc_action_difference");
  return ds;
}

void GpuCompositeAction::getBeadAction(const Paths&, int, int, double&, double&, double&, Vec&,
                                       Vec&) const {
  throw std::runtime_error("GpuCompositeAction: per-bead actions run in gpuThermoEnergy");
}

GpuNodeModel::GpuNodeModel(pimc_engine* engine, int ispec, int npart)
    : NodeModel("_gpu"), engine(engine), ispec(ispec), npart(npart),
      r1buf(3 * npart), r2buf(3 * npart), d1buf(npart), d2buf(npart) {}

NodeModel::DetWithFlag GpuNodeModel::evaluate(const VArray& r1, const VArray& r2, const int,
                                              bool) {
  for (int i = 0; i < npart; ++i)
    for (int d = 0; d < 3; ++d) {
      r1buf[3 * i + d] = r1(i)[d];
      r2buf[3 * i + d] = r2(i)[d];
    }
  DetWithFlag res;
  int err = 0;
  check(pimc_node_evaluate(engine, ispec, 1, &r1buf[0], &r2buf[0], &res.det, &d1buf[0],
                           &d2buf[0], &err),
        "pimc_node_evaluate");
  res.err = err != 0;
  return res;
}

void GpuNodeModel::evaluateDistance(const VArray&, const VArray&, const int, Array& d1,
                                    Array& d2) {
  // Distances of the slice pair passed to the preceding evaluate().
  for (int i = 0; i < npart; ++i) {
    d1(i) = d1buf[i];
    d2(i) = d2buf[i];
  }
}

GpuSectionSampler::GpuSectionSampler(Paths& paths, pimc_engine* engine, int attempts)
    : paths(paths), engine(engine), attempts(attempts),
      host(3 * (size_t)paths.getNPart() * paths.getNSlice()) {}

void GpuSectionSampler::run() {
  const int np = paths.getNPart(), ns = paths.getNSlice();
  for (int t = 0; t < ns; ++t)
    for (int i = 0; i < np; ++i)
      for (int d = 0; d < 3; ++d) host[(t * np + i) * 3 + d] = paths(i, t)[d];
  check(pimc_upload_paths(engine, &host[0]), "pimc_upload_paths");
  check(pimc_run_sections(engine, attempts, 0), "pimc_run_sections");
  check(pimc_download_paths(engine, &host[0]), "pimc_download_paths");
  for (int t = 0; t < ns; ++t)
    for (int i = 0; i < np; ++i)
      for (int d = 0; d < 3; ++d) paths(i, t)[d] = host[(t * np + i) * 3 + d];
}

double gpuThermoEnergy(const Paths& paths, pimc_engine* engine) {
  const int np = paths.getNPart(), ns = paths.getNSlice();
  std::vector<double> host(3 * (size_t)np * ns);
  for (int t = 0; t < ns; ++t)
    for (int i = 0; i < np; ++i)
      for (int d = 0; d < 3; ++d) host[(t * np + i) * 3 + d] = paths(i, t)[d];
  check(pimc_upload_paths(engine, &host[0]), "pimc_upload_paths");
  double e = 0;
  check(pimc_thermo_energy(engine, &e), "pimc_thermo_energy");
  return e;
}

pimc_system systemFromSimulation(const SimulationInfo& simInfo, const SystemOptions& opt) {
  pimc_system sys;
  memset(&sys, 0, sizeof(sys));
  sys.npart = simInfo.getNPart();
  sys.nspecies = simInfo.getNSpecies();
  if (sys.nspecies > PIMC_MAX_SPECIES) throw std::runtime_error("too many species");
  for (int i = 0; i < sys.nspecies; ++i) {
    const Species& sp = simInfo.getSpecies(i);
    sys.spec_count[i] = sp.count;
    sys.spec_mass[i] = sp.mass;
    sys.spec_charge[i] = sp.charge;
    sys.sho_omega[i] = i < (int)opt.sho_omega.size() ? opt.sho_omega[i] : 0.0;
    sys.node_kind[i] = i < (int)opt.node_kind.size() ? opt.node_kind[i] : PIMC_NODES_NONE;
    sys.node_omega[i] = i < (int)opt.node_omega.size() ? opt.node_omega[i] : 0.0;
  }
  sys.node_temperature = opt.node_temperature > 0 ? opt.node_temperature : simInfo.getTemperature();
  sys.nslice = simInfo.getNSlice();
  sys.tau = simInfo.getTau();
  sys.nlevel = opt.nlevel;
  const SuperCell& cell = *simInfo.getSuperCell();
  for (int d = 0; d < NDIM; ++d) sys.cell[d] = cell[d];
  sys.spring = opt.spring ? 1 : 0;
  sys.coulomb = opt.coulomb ? 1 : 0;
  sys.epsilon = opt.epsilon;
  sys.ewald = opt.ewald ? 1 : 0;
  sys.mover = opt.pbc_mover ? PIMC_MOVER_FREE_PBC : PIMC_MOVER_FREE;
  return sys;
}

}  // namespace pimc_gb300
