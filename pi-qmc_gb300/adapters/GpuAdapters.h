// Adapters that put the GB300 engine (include/pimc_gb300.h) behind pi-qmc's own
// interfaces, so pi-qmc's samplers, estimators and parsers can use it unchanged.
// They compile against pi-qmc's headers (src/ and contrib/blitz-0.9) and link
// against libpimc_gb300.so; they are the pi-qmc side of the integration.
//
//   GpuCompositeAction : Action      getActionDifference offloaded
//                                    (replaces CompositeAction, src/action/CompositeAction.h)
//   GpuNodeModel       : NodeModel   evaluate / evaluateDistance offloaded
//                                    (replaces SHONodes / FreeParticleNodes)
//   GpuSectionSampler  : Algorithm   whole section moves on the device
//                                    (replaces SectionChooser + MultiLevelSampler /
//                                     DoubleSectionChooser + DoubleMLSampler)
//   gpuThermoEnergy()                ThermoEnergyEstimator's value on the device
//
// Every engine error is raised as std::runtime_error carrying pimc_last_error():
// there is no CPU fallback.
#ifndef PIMC_GB300_ADAPTERS_H
#define PIMC_GB300_ADAPTERS_H

#include <vector>

#include "action/Action.h"
#include "algorithm/Algorithm.h"
#include "fixednode/NodeModel.h"
#include "pimc_gb300.h"

class Paths;
class SectionSamplerInterface;
class SimulationInfo;

namespace pimc_gb300 {

// Throws std::runtime_error for a nonzero engine status.
void check(int status, const char* what);

// Action offload: CompositeAction::getActionDifference for one moving particle
// (src/action/CompositeAction.cc:30-37).  The engine must describe the same
// system as the actions it replaces (spring, SHO, PrimSHO, Coulomb tables).
class GpuCompositeAction : public Action {
 public:
  GpuCompositeAction(pimc_engine* engine, int npart, int nlevel);
  virtual double getActionDifference(const SectionSamplerInterface&, int level);
  virtual double getTotalAction(const Paths&, const int level) const { return 0; }
  // Per-bead actions are not offloaded one bead at a time; use gpuThermoEnergy.
  virtual void getBeadAction(const Paths&, int ipart, int islice, double& u, double& utau,
                             double& ulambda, Vec& fm, Vec& fp) const;

 private:
  pimc_engine* engine;
  int npart, nsec;
  std::vector<double> section, moving;
};

// NodeModel offload for one species (NodeModel::evaluate / evaluateDistance,
// src/fixednode/NodeModel.h:74-90).  The engine's current scale for the
// species is used; set-up rescaling happens in GpuSectionSampler.
class GpuNodeModel : public NodeModel {
 public:
  GpuNodeModel(pimc_engine* engine, int ispec, int npart);
  virtual DetWithFlag evaluate(const VArray& r1, const VArray& r2, const int islice,
                               bool scaleMagnitude);
  virtual void evaluateDistance(const VArray& r1, const VArray& r2, const int islice,
                                Array& d1, Array& d2);
  virtual void evaluateGradLogDist(const VArray&, const VArray&, const int, VMatrix&,
                                   VMatrix&, const Array&, const Array&) {}

 private:
  pimc_engine* engine;
  int ispec, npart;
  std::vector<double> r1buf, r2buf, d1buf, d2buf;
};

// Sampler offload: each run() performs `attempts` section-move attempts of
// pi-qmc's bisection sampler on the device for the engine's replica 0, with the
// paths copied in from and back to pi-qmc's Paths.
class GpuSectionSampler : public Algorithm {
 public:
  GpuSectionSampler(Paths& paths, pimc_engine* engine, int attempts);
  virtual void run();

 private:
  Paths& paths;
  pimc_engine* engine;
  int attempts;
  std::vector<double> host;
};

// ThermoEnergyEstimator's value (src/estimator/ThermoEnergyEstimator.cc:32-66)
// for pi-qmc's current paths, computed on the device.
double gpuThermoEnergy(const Paths& paths, pimc_engine* engine);

// The attributes pi-qmc's parsers read for the actions, node models and
// sampler of this path (src/parser/ActionParser.cc:105-153,433-452,
// src/parser/PIMCParser.cc:312-491) that SimulationInfo does not hold.
struct SystemOptions {
  int nlevel = 5;                  // <Sample nlevel=...>
  bool spring = true;              // <SpringAction/>
  bool coulomb = false;            // <CoulombAction/> (pair tables needed)
  bool ewald = false;              // <CoulombAction ewald="true"/> (Ewald table needed)
  bool pbc_mover = false;          // FreeMoverPBC instead of FreeMover
  double epsilon = 1.0;            // dielectric constant
  std::vector<double> sho_omega;   // <SHOAction omega=...> per species (empty or 0: none)
  std::vector<int> node_kind;      // PIMC_NODES_* per species (<FixedNodeAction model=...>)
  std::vector<double> node_omega;  // SHONodes omega per species
  double node_temperature = 0;     // trial density matrix temperature (0: the simulation's)
};

// The engine's description of pi-qmc's system: species, masses and charges,
// slices, tau and cell from SimulationInfo, the rest from the options.
pimc_system systemFromSimulation(const SimulationInfo& simInfo, const SystemOptions& opt);

}  // namespace pimc_gb300
#endif
