// Reads a <GpuAction> fragment with the GPU tag parser (GpuParser.cc, on
// pi-qmc's own XMLParser helpers) for a simulation pi-qmc's objects describe,
// and prints the engine system it yields, then builds a <GpuSample> sampler.
// TEST INFRASTRUCTURE for tests/test_adapters.py; libxml2 is replaced by the
// stand-in headers beside this file.
#include <cstdio>
#include <stdexcept>

#include "GpuParser.h"
#include "oracle_api.h"

extern "C" {
void* ref_create(const ora_config* c);
void* ref_paths(void* h);
void* ref_simulation_info(void* h);
}

static xmlNode elem(const char* name, const char* const* attrs, xmlNode* children = 0,
                    xmlNode* next = 0) {
  xmlNode n;
  n.type = XML_ELEMENT_NODE;
  n.name = BAD_CAST name;
  n.children = children;
  n.next = next;
  n.attrs = attrs;
  return n;
}

int main() {
  // the small fixed-node dot: 2 up + 2 down electrons, M = 64, beta = 4
  ora_config c = ora_config();
  c.npart = 4;
  c.nspecies = 2;
  for (int i = 0; i < 2; ++i) {
    c.spec_count[i] = 2;
    c.spec_mass[i] = 1.0;
    c.spec_charge[i] = -1.0;
  }
  c.nslice = 64;
  c.tau = 4.0 / 64;
  c.temperature = 0.25;
  c.node_temperature = 0.25;
  c.nlevel = 3;
  for (int d = 0; d < 3; ++d) c.cell[d] = 1000.0;
  c.spring = 1;
  c.epsilon = 1.0;
  c.norder = 3;
  void* h = ref_create(&c);
  const SimulationInfo& si = *(const SimulationInfo*)ref_simulation_info(h);

  static const char* const fna[] = {"species", "dn", "model", "SHONodes", "omega", "1.5", 0};
  static const char* const fua[] = {"species", "up", "model", "SHONodes", "omega", "1.25",
                                    "temperature", "0.5", 0};
  static const char* const ca[] = {"norder", "3", "epsilon", "2", 0};
  static const char* const pa[] = {"species", "dn", "a", "0.5", "b", "0.25", 0};
  static const char* const sa[] = {"omega", "1", 0};
  static const char* const ga[] = {"nlevel", "3", "mover", "Free", "precision", "mixed",
                                   "replicas", "7", "delayedRejection", "true",
                                   "newSigmaFactor", "0.6", 0};
  static const char* const none[] = {0};
  xmlNode fn_dn = elem("FixedNodeAction", fna);
  xmlNode fn_up = elem("FixedNodeAction", fua, 0, &fn_dn);
  xmlNode coul = elem("CoulombAction", ca, 0, &fn_up);
  xmlNode prim = elem("PrimSHOAction", pa, 0, &coul);
  xmlNode sho = elem("SHOAction", sa, 0, &prim);
  xmlNode spring = elem("SpringAction", none, 0, &sho);
  xmlNode gpu = elem("GpuAction", ga, &spring);

  pimc_gb300::GpuActionSpec spec = pimc_gb300::GpuParser::parseAction(&gpu, si);
  pimc_system s = pimc_gb300::GpuParser::system(spec, si);
  printf("%d %d %d %d %g %g %g %g %g %g %g %g %d %d %g %g %g %d %.17g %d %g %d %d %g %d %d\n",
         s.npart, s.nspecies, s.spec_count[0], s.spec_count[1], s.sho_omega[0], s.sho_omega[1],
         s.prim_a[0], s.prim_a[1], s.prim_b[1], s.spec_mass[0], s.spec_charge[1], s.cell[0],
         s.node_kind[0], s.node_kind[1], s.node_omega[0], s.node_omega[1], s.node_temperature,
         s.nslice, s.tau, s.nlevel, s.epsilon, s.spring, s.coulomb, (double)spec.norder, s.mover,
         spec.replicas);
  printf("%d\n", spec.precision);
  printf("%d %g %g\n", s.delayed_rejection, s.sigma_factor, s.dr_sigma_factor);

  // an unknown child and a mover that disagrees are refused
  xmlNode bad = elem("EwaldAction", none);
  xmlNode gbad = elem("GpuAction", none, &bad);
  int refused = 0;
  try {
    pimc_gb300::GpuParser::parseAction(&gbad, si);
  } catch (const std::runtime_error&) {
    refused += 1;
  }
  static const char* const sma[] = {"attempts", "640", "mover", "FreePBC", 0};
  xmlNode smp = elem("GpuSample", sma);
  try {
    pimc_gb300::GpuParser::parseSample(&smp, *(Paths*)ref_paths(h), 0, spec);
  } catch (const std::runtime_error&) {
    refused += 1;
  }
  static const char* const smd[] = {"attempts", "640", "delayedRejection", "false", 0};
  xmlNode smpd = elem("GpuSample", smd);
  try {
    pimc_gb300::GpuParser::parseSample(&smpd, *(Paths*)ref_paths(h), 0, spec);
  } catch (const std::runtime_error&) {
    refused += 1;
  }
  static const char* const smb[] = {"attempts", "640", "delayedRejection", "true", 0};
  xmlNode smp2 = elem("GpuSample", smb);
  Algorithm* a = pimc_gb300::GpuParser::parseSample(&smp2, *(Paths*)ref_paths(h), 0, spec);
  printf("%d %d\n", refused, a != 0);
  return 0;
}
