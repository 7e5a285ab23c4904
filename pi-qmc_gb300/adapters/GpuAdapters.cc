#include "GpuAdapters.h"

#include <cmath>
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
  throw std::logic_error(
      "GpuCompositeAction::getBeadAction: per-bead actions are summed on the device "
      "(gpuThermoEnergy, pimc_virial_energy)");
}

GpuNodeModel::GpuNodeModel(pimc_engine* engine, int ispec, int npart, int count, int maxlevel)
    : NodeModel("_gpu"), engine(engine), ispec(ispec), npart(npart), count(count), scale(1.0),
      slices((1 << maxlevel) + 1), r1buf(3 * npart), r2buf(3 * npart) {
  for (size_t k = 0; k < slices.size(); ++k) slices[k].valid = false;
  pushScale();
}

// The engine evaluates at its replica-0 scale for the species: keep it this model's.
void GpuNodeModel::pushScale() {
  pimc_replica_state st;
  check(pimc_get_replica_state(engine, 0, &st), "pimc_get_replica_state");
  if (st.node_scale[ispec] == scale) return;
  st.node_scale[ispec] = scale;
  check(pimc_set_replica_state(engine, 0, &st), "pimc_set_replica_state");
}

void GpuNodeModel::pack(const VArray& r1, const VArray& r2) {
  for (int i = 0; i < npart; ++i)
    for (int d = 0; d < 3; ++d) {
      r1buf[3 * i + d] = r1(i)[d];
      r2buf[3 * i + d] = r2(i)[d];
    }
}

GpuNodeModel::SliceResult& GpuNodeModel::slot(int islice) {
  if (islice < 0) throw std::out_of_range("GpuNodeModel: negative slice index");
  if (islice >= (int)slices.size()) {
    const size_t old = slices.size();
    slices.resize(islice + 1);
    for (size_t k = old; k < slices.size(); ++k) slices[k].valid = false;
  }
  return slices[islice];
}

// One evaluation of the packed positions at the current scale, kept for islice.
NodeModel::DetWithFlag GpuNodeModel::evaluateOnce(int islice) {
  SliceResult& r = slot(islice);
  r.d1.resize(npart);
  r.d2.resize(npart);
  DetWithFlag res;
  int err = 0;
  check(pimc_node_evaluate(engine, ispec, 1, &r1buf[0], &r2buf[0], &res.det, &r.d1[0],
                           &r.d2[0], &err),
        "pimc_node_evaluate");
  res.err = err != 0;
  r.det = res.det;
  r.r1 = r1buf;
  r.r2 = r2buf;
  r.valid = true;
  return res;
}

NodeModel::DetWithFlag GpuNodeModel::evaluate(const VArray& r1, const VArray& r2,
                                              const int islice, bool scaleMagnitude) {
  pack(r1, r2);
  DetWithFlag res = evaluateOnce(islice);
  // SHONodes::evaluate's rescale loop (src/fixednode/SHONodes.cc:53-126)
  for (int guard = 0; scaleMagnitude && !res.err &&
                      (std::fabs(res.det) < 1e-50 || std::fabs(res.det) > 1e50);
       ++guard) {
    if (guard >= 2000) throw std::runtime_error("GpuNodeModel: rescale loop did not converge");
    if (std::fabs(res.det) < 1e-250)
      scale *= 2;
    else
      scale *= std::pow(std::fabs(res.det), -1. / count);
    pushScale();
    res = evaluateOnce(islice);
  }
  return res;
}

void GpuNodeModel::evaluateDistance(const VArray& r1, const VArray& r2, const int islice,
                                    Array& d1, Array& d2) {
  pack(r1, r2);
  SliceResult& r = slot(islice);
  if (!r.valid || r.r1 != r1buf || r.r2 != r2buf) evaluateOnce(islice);
  for (int i = 0; i < npart; ++i) {
    d1(i) = r.d1[i];
    d2(i) = r.d2[i];
  }
}

void GpuNodeModel::evaluateGradLogDist(const VArray&, const VArray&, const int, VMatrix&,
                                       VMatrix&, const Array&, const Array&) {
  throw std::logic_error("GpuNodeModel::evaluateGradLogDist is not offloaded");
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
