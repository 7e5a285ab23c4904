// The XML front end of the GPU path: the tags a pi-qmc input uses to run its
// bisection sampler, actions and node models on the engine.  They compile
// against pi-qmc's parser headers (src/parser/XMLParser.h, libxml2) and are
// called from pi-qmc's own parsers, which a maintainer extends by two branches
// (INTEGRATION.md shows them):
//
//   <Action>                                   ActionParser::parse (src/parser/ActionParser.cc:105-153)
//     <GpuAction nlevel="5" mover="FreePBC" precision="mixed" replicas="1" seed="20261203"
//                delayedRejection="false" defaultSigmaFactor="1" newSigmaFactor="0.75">
//       <SpringAction/>                        the usual pi-qmc action tags, with their
//       <SHOAction omega="1" species="up"/>    own attribute names (ActionParser.cc:110-200,
//       <PrimSHOAction a="0.5" b="0.1"/>       307-320, 433-452, 760-790); a tag without
//       <CoulombAction norder="3" useEwald="false"/>   `species` applies to every species
//       <FixedNodeAction species="up" model="SHONodes" omega="1" temperature="0.05"/>
//     </GpuAction>
//   </Action>
//   <GpuSample attempts="640" mover="Free"/>   PIMCParser::parseAlgorithm (src/parser/PIMCParser.cc:312-494)
//
// Numbers are read in the simulation's internal units (Hartree, bohr); unit
// suffixes are not converted.  Node models: SHONodes and FreeParticleNodes.
// The bisection mover and the sampler's width factors and delayed rejection
// are part of the engine, so they are named on <GpuAction> (`mover`, "Free" or
// "FreePBC", pi-qmc's default; `delayedRejection`, `defaultSigmaFactor`,
// `newSigmaFactor`, pi-qmc's <Sample> attribute names) rather than on the
// sampler; a <GpuSample> that repeats one of them must agree.
#ifndef PIMC_GB300_GPU_PARSER_H
#define PIMC_GB300_GPU_PARSER_H

#include <string>
#include <vector>

#include "GpuAdapters.h"
#include "parser/XMLParser.h"

namespace pimc_gb300 {

// What a <GpuAction> element and its children say, beside SimulationInfo.
struct GpuActionSpec {
  SystemOptions opt;
  std::vector<double> prim_a, prim_b;  // PrimSHOAction per species
  int norder = 3;                      // CoulombAction norder
  double ewald_rcut = 0, ewald_kcut = 0;
  int precision = PIMC_PREC_FP64;
  // the bisection sampler's <Sample> attributes (src/parser/PIMCParser.cc:312-322):
  // delayedRejection, defaultSigmaFactor, newSigmaFactor (0: pi-qmc's defaults)
  bool delayed_rejection = false;
  double sigma_factor = 0, dr_sigma_factor = 0;
  int replicas = 1;
  unsigned long long seed = 20261203ull;
};

class GpuParser : public XMLParser {
 public:
  // Reads a <GpuAction> element: its attributes and its pi-qmc action children.
  // Unknown children or node models throw std::runtime_error.
  static GpuActionSpec parseAction(const xmlNodePtr& gpuAction, const SimulationInfo& simInfo);
  // The engine's system description for that element (species, slices, tau
  // and cell from SimulationInfo).
  static pimc_system system(const GpuActionSpec& spec, const SimulationInfo& simInfo);
  // Builds the engine, with the pair and Ewald tables the engine's builder
  // makes (pimc_coulomb_tables reproduces CoulombAction's to 7e-15 relative).
  static pimc_engine* createEngine(const GpuActionSpec& spec, const SimulationInfo& simInfo);
  // <GpuSample attempts=.. mover="Free|FreePBC">: the device sampler.  The
  // mover and the sampler attributes are fixed when the engine is built, so a
  // `mover` or `delayedRejection` that disagrees with the GpuAction's throws.
  static Algorithm* parseSample(const xmlNodePtr& gpuSample, Paths& paths, pimc_engine* engine,
                                const GpuActionSpec& spec);

 private:
  static int speciesIndex(const SimulationInfo& simInfo, const std::string& name);
};

}  // namespace pimc_gb300
#endif
