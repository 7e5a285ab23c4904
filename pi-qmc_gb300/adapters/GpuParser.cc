#include "GpuParser.h"

#include <stdexcept>

#include "base/SimulationInfo.h"
#include "base/Species.h"

namespace pimc_gb300 {

int GpuParser::speciesIndex(const SimulationInfo& simInfo, const std::string& name) {
  for (int i = 0; i < simInfo.getNSpecies(); ++i)
    if (simInfo.getSpecies(i).name == name) return i;
  throw std::runtime_error("GpuAction: no species named " + name);
}

GpuActionSpec GpuParser::parseAction(const xmlNodePtr& gpu, const SimulationInfo& simInfo) {
  GpuActionSpec spec;
  const int ns = simInfo.getNSpecies();
  SystemOptions& o = spec.opt;
  o.spring = false;
  o.sho_omega.assign(ns, 0.0);
  o.node_kind.assign(ns, PIMC_NODES_NONE);
  o.node_omega.assign(ns, 0.0);
  spec.prim_a.assign(ns, 0.0);
  spec.prim_b.assign(ns, 0.0);
  const int nlevel = getIntAttribute(gpu, "nlevel");
  if (nlevel > 0) o.nlevel = nlevel;
  const std::string prec = getStringAttribute(gpu, "precision");
  if (prec == "mixed")
    spec.precision = PIMC_PREC_MIXED;
  else if (prec != "" && prec != "fp64")
    throw std::runtime_error("GpuAction: precision is fp64 or mixed");
  const int nrep = getIntAttribute(gpu, "replicas");
  if (nrep > 0) spec.replicas = nrep;
  const std::string seed = getStringAttribute(gpu, "seed");
  if (seed != "") spec.seed = std::stoull(seed);
  o.pbc_mover = getStringAttribute(gpu, "mover") != "Free";  // pi-qmc's default is FreePBC
  spec.delayed_rejection = getBoolAttribute(gpu, "delayedRejection");
  spec.sigma_factor = getDoubleAttribute(gpu, "defaultSigmaFactor");
  spec.dr_sigma_factor = getDoubleAttribute(gpu, "newSigmaFactor");
  for (xmlNodePtr c = gpu->children; c; c = c->next) {
    if (c->type != XML_ELEMENT_NODE) continue;
    const std::string name = getName(c);
    // the species a tag applies to: the one named, or all of them
    const std::string spn = getStringAttribute(c, "species");
    const int lo = spn == "" ? 0 : speciesIndex(simInfo, spn);
    const int hi = spn == "" ? ns : lo + 1;
    if (name == "SpringAction") {
      o.spring = true;
    } else if (name == "SHOAction") {
      double omega = getDoubleAttribute(c, "omega");
      if (omega == 0) omega = 1;  // ActionParser's default
      for (int i = lo; i < hi; ++i) o.sho_omega[i] = omega;
    } else if (name == "PrimSHOAction") {
      for (int i = lo; i < hi; ++i) {
        spec.prim_a[i] = getDoubleAttribute(c, "a");
        spec.prim_b[i] = getDoubleAttribute(c, "b");
      }
    } else if (name == "CoulombAction") {
      o.coulomb = true;
      o.epsilon = getDoubleAttribute(c, "epsilon");
      if (o.epsilon == 0) o.epsilon = 1;
      const int norder = getIntAttribute(c, "norder");
      if (norder > 0) spec.norder = norder;
      o.ewald = getBoolAttribute(c, "useEwald");
      spec.ewald_rcut = getDoubleAttribute(c, "ewaldRcut");
      spec.ewald_kcut = getDoubleAttribute(c, "ewaldKcut");
    } else if (name == "FixedNodeAction") {
      const std::string model = getStringAttribute(c, "model");
      int kind = PIMC_NODES_NONE;
      if (model == "SHONodes")
        kind = PIMC_NODES_SHO;
      else if (model == "FreeParticleNodes")
        kind = PIMC_NODES_FREE;
      else
        throw std::runtime_error("GpuAction: node model " + model + " is not on the device");
      const double t = getDoubleAttribute(c, "temperature");
      if (t > 0) o.node_temperature = t;
      for (int i = lo; i < hi; ++i) {
        o.node_kind[i] = kind;
        o.node_omega[i] = kind == PIMC_NODES_SHO ? getDoubleAttribute(c, "omega") : 0.0;
      }
    } else {
      throw std::runtime_error("GpuAction: " + name + " is not on the device");
    }
  }
  return spec;
}

pimc_system GpuParser::system(const GpuActionSpec& spec, const SimulationInfo& simInfo) {
  pimc_system sys = systemFromSimulation(simInfo, spec.opt);
  for (int i = 0; i < sys.nspecies; ++i) {
    sys.prim_a[i] = spec.prim_a[i];
    sys.prim_b[i] = spec.prim_b[i];
  }
  sys.delayed_rejection = spec.delayed_rejection ? 1 : 0;
  sys.sigma_factor = spec.sigma_factor;
  sys.dr_sigma_factor = spec.dr_sigma_factor;
  return sys;
}

pimc_engine* GpuParser::createEngine(const GpuActionSpec& spec, const SimulationInfo& simInfo) {
  const pimc_system sys = system(spec, simInfo);
  const pimc_pair_table* tabs = 0;
  const pimc_ewald_table* ew = 0;
  int ntab = 0;
  if (sys.coulomb)
    check(pimc_coulomb_tables(&sys, spec.norder, 0, 0.0, 0.0, spec.ewald_rcut, spec.ewald_kcut,
                              &tabs, &ntab, &ew),
          "pimc_coulomb_tables");
  pimc_engine* e = 0;
  check(pimc_engine_create(&sys, spec.replicas, tabs, ntab, sys.ewald ? ew : 0, spec.seed,
                           spec.precision, &e),
        "pimc_engine_create");
  return e;
}

Algorithm* GpuParser::parseSample(const xmlNodePtr& node, Paths& paths, pimc_engine* engine,
                                  const GpuActionSpec& spec) {
  const std::string mover = getStringAttribute(node, "mover");
  if (mover != "" && (mover == "Free") == spec.opt.pbc_mover)
    throw std::runtime_error("GpuSample: mover differs from the GpuAction's");
  if (getStringAttribute(node, "delayedRejection") != "" &&
      getBoolAttribute(node, "delayedRejection") != spec.delayed_rejection)
    throw std::runtime_error("GpuSample: delayedRejection differs from the GpuAction's");
  int attempts = getIntAttribute(node, "attempts");
  if (attempts <= 0) attempts = 1;
  return new GpuSectionSampler(paths, engine, attempts);
}

}  // namespace pimc_gb300
