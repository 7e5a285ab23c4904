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
  // Every action this one replaces returns 0 here (SpringAction.cc:108-110,
  // SHOAction.cc:67-69, PrimSHOAction.cc:60-63, CoulombAction.cc:150-152,
  // PairAction.cc:505-507 in src/action), so their composite does too.
  virtual double getTotalAction(const Paths&, const int level) const { return 0; }
  // Per-bead actions are not offloaded one bead at a time: the estimators'
  // sums over links run on the device (gpuThermoEnergy, pimc_virial_energy).
  // A call throws std::logic_error rather than returning wrong values.
  virtual void getBeadAction(const Paths&, int ipart, int islice, double& u, double& utau,
                             double& ulambda, Vec& fm, Vec& fp) const;

 private:
  pimc_engine* engine;
  int npart, nsec;
  std::vector<double> section, moving;
};

// NodeModel offload for one species (NodeModel::evaluate / evaluateDistance,
// src/fixednode/NodeModel.h:74-90), holding what SHONodes / FreeParticleNodes
// hold per section slice (src/fixednode/SHONodes.cc:51-170): evaluate(r1, r2,
// islice) keeps that slice's determinant and nodal distances, and
// evaluateDistance(r1, r2, islice) returns them when r1, r2 are the positions
// last evaluated on islice (FixedNodeAction's order: every slice is evaluated
// at its level before the level-0 distances, src/fixednode/FixedNodeAction.cc:58-100),
// else evaluates those positions.  The model's scale starts at 1 and follows
// pi-qmc's rescale loop when evaluate is asked to scale the magnitude
// (|det| outside [1e-50, 1e50]: scale *= 2 below 1e-250, else |det|^(-1/n));
// the engine's replica-0 scale for the species is kept equal to it, so the
// device builds scale * rho exactly as pi-qmc does.  A singular matrix with
// scaleMagnitude returns err = true instead of pi-qmc's retry-until-exit.
class GpuNodeModel : public NodeModel {
 public:
  // npart: all particles; count: the species' particles (SHONodes' npart);
  // maxlevel: the bisection level (slices 0 .. 2^maxlevel kept, as SHONodes).
  GpuNodeModel(pimc_engine* engine, int ispec, int npart, int count, int maxlevel);
  virtual DetWithFlag evaluate(const VArray& r1, const VArray& r2, const int islice,
                               bool scaleMagnitude);
  virtual void evaluateDistance(const VArray& r1, const VArray& r2, const int islice,
                                Array& d1, Array& d2);
  // Not offloaded; pi-qmc's FixedNodeAction does not call it (SHONodes' own is
  // empty).  A call throws std::logic_error.
  virtual void evaluateGradLogDist(const VArray&, const VArray&, const int, VMatrix&,
                                   VMatrix&, const Array&, const Array&);
  double getScale() const { return scale; }

 private:
  struct SliceResult {
    bool valid;
    double det;
    std::vector<double> r1, r2, d1, d2;
  };
  pimc_engine* engine;
  int ispec, npart, count;
  double scale;
  std::vector<SliceResult> slices;
  std::vector<double> r1buf, r2buf;
  void pack(const VArray& r1, const VArray& r2);
  SliceResult& slot(int islice);
  DetWithFlag evaluateOnce(int islice);
  void pushScale();
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
