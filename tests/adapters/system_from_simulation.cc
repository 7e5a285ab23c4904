// Builds a pi-qmc SimulationInfo (two species in a 10 x 11 x 12 cell) and
// prints the engine description pimc_gb300::systemFromSimulation makes of it;
// compiled and run by tests/test_adapters.py against pi-qmc's own objects.
#include "config.h"
#include <cstdio>
#include <vector>
#include "GpuAdapters.h"
#include "base/SimulationInfo.h"
#include "base/Species.h"
#include "util/SuperCell.h"
int main() {
  SuperCell* cell = new SuperCell(SuperCell::Vec(10.0, 11.0, 12.0));
  std::vector<Species*> specs, index;
  specs.push_back(new Species("up", 2, 1.0, -1.0, 1, true));
  specs.push_back(new Species("dn", 3, 2.0, 1.0, 1, true));
  specs[1]->ifirst = 2;
  for (int i = 0; i < 5; ++i) index.push_back(specs[i < 2 ? 0 : 1]);
  SimulationInfo si(cell, 5, specs, index, 0.5, 0.05, 40);
  pimc_gb300::SystemOptions o;
  o.nlevel = 3; o.coulomb = true; o.pbc_mover = true;
  o.sho_omega.push_back(1.0); o.sho_omega.push_back(2.0);
  o.node_kind.push_back(PIMC_NODES_SHO); o.node_kind.push_back(PIMC_NODES_FREE);
  o.node_omega.push_back(1.5);
  pimc_system s = pimc_gb300::systemFromSimulation(si, o);
  printf("%d %d %d %d %g %g %g %g %g %g %d %d %g %g %d %g %d %g %g %g %d %d %d %d\n", s.npart, s.nspecies,
         s.spec_count[0], s.spec_count[1], s.spec_mass[0], s.spec_mass[1], s.spec_charge[0],
         s.spec_charge[1], s.sho_omega[0], s.sho_omega[1], s.node_kind[0], s.node_kind[1],
         s.node_omega[0], s.node_omega[1], s.nslice, s.tau, s.nlevel, s.cell[0], s.cell[1], s.cell[2],
         s.spring, s.coulomb, s.ewald, s.mover);
  printf("%g\n", s.node_temperature);
  return 0;
}
