// Driver for pi-qmc's own hot-path objects, compiled with them into
// oracle/_ref/libpimcref.so by oracle/build_ref.py.  TEST INFRASTRUCTURE:
// it builds SimulationInfo / SerialPaths / CompositeAction / FixedNodeAction /
// samplers directly (what src/parser/ActionParser.cc:105-153,433-452 and
// src/parser/PIMCParser.cc:312-491 would build from XML, with their defaults),
// runs section moves on random numbers served by the replay shim, and records
// per-level action differences, mover log transition ratios and decisions.
#include "config.h"
#include <blitz/array.h>
#include <blitz/tinyvec-et.h>
#include <cmath>
#include <complex>
#include <cstdio>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

// Read access to the reference objects' tables (pair-action grids, Ewald
// k-vectors, node-model scale) for export to the tests.
#define private public
#define protected public
#include "action/Action.h"
#include "action/CompositeAction.h"
#include "action/CompositeDoubleAction.h"
#include "action/CoulombAction.h"
#include "action/DoubleAction.h"
#include "action/PairAction.h"
#include "action/PrimSHOAction.h"
#include "action/SHOAction.h"
#include "action/SpringAction.h"
#include "advancer/DoubleMLSampler.h"
#include "advancer/DoubleSectionChooser.h"
#include "advancer/MultiLevelSampler.h"
#include "advancer/PermutationChooser.h"
#include "advancer/SectionChooser.h"
#include "advancer/SectionSamplerInterface.h"
#include "advancer/SimpleParticleChooser.h"
#include "advancer/mover/FreeMover.h"
#include "advancer/mover/FreeMoverPBC.h"
#include "advancer/mover/Mover.h"
#include "base/BeadFactory.h"
#include "base/Beads.h"
#include "base/LinkSummable.h"
#include "base/SerialPaths.h"
#include "base/SimulationInfo.h"
#include "base/Species.h"
#include "fixednode/FixedNodeAction.h"
#include "fixednode/FreeParticleNodes.h"
#include "fixednode/NodeModel.h"
#include "fixednode/SHONodes.h"
#include "util/EwaldSum.h"
#include "util/OptEwaldSum.h"
#include "util/SuperCell.h"
#include "algorithm/PathReader.h"
#include "algorithm/WritePaths.h"
#undef private
#undef protected

#include "../pi-qmc_gb300/csrc/pimc_rng.h"
#include "oracle_api.h"

typedef blitz::TinyVector<double, NDIM> Vec;

// ---- random-number replay -------------------------------------------------
static uint64_t g_seed = 0;
static uint32_t g_replica = 0, g_attempt = 0, g_uidx = 0, g_npair = 0;

static void shim_begin_attempt(uint64_t seed, uint32_t replica, uint32_t attempt) {
  g_seed = seed;
  g_replica = replica;
  g_attempt = attempt;
  g_uidx = 0;
  g_npair = 0;
}

extern "C" double oracle_shim_uniform(void) {
  return pimc::stream_uniform(g_seed, g_replica, g_attempt, g_uidx++);
}

extern "C" void oracle_shim_normals(double* out, int n) {
  for (int i = 0; i < n; i += 2) {
    double z0, z1;
    pimc::stream_normal_pair(g_seed, g_replica, g_attempt, g_npair++, &z0, &z1);
    out[i] = z0;
    if (i + 1 < n) out[i + 1] = z1;
  }
}

// Unused on the bisection path; defined so the objects link.
#include "action/interaction/PairIntegrator.h"
#include "stats/ReportWriters.h"
#include <cstring>
#define protected public
#include "advancer/DisplaceMoveSampler.h"
#include "advancer/DoubleDisplaceMoveSampler.h"
#undef protected
#include "advancer/UniformMover.h"
#include "advancer/SpeciesParticleChooser.h"
#include "estimator/VirialEnergyEstimator.h"
#include "estimator/CoulombEnergyEstimator.h"
#include "estimator/EwaldCoulombEstimator.h"
#include "stats/SimpleScalarAccumulator.h"
void PairIntegrator::integrate(double, double) {}
void ReportWriters::startAccRejReport(AccRejEstimator*, ScalarAccumulator*) {}
void ReportWriters::reportAccRejStep(AccRejEstimator*, ScalarAccumulator*) {}
void ReportWriters::startScalarReport(ScalarEstimator*, SimpleScalarAccumulator*) {}
void ReportWriters::reportScalarStep(ScalarEstimator*, SimpleScalarAccumulator*) {}
void ReportWriters::startScalarReport(ScalarEstimator*, PartitionedScalarAccumulator*) {}
void ReportWriters::reportScalarStep(ScalarEstimator*, PartitionedScalarAccumulator*) {}


// ---- recording wrappers ---------------------------------------------------
static ora_record* g_rec = 0;
static ora_drecord* g_drec = 0;
static bool g_accepted = false;
static int g_lowest_level = 99;

class RecAction : public Action {
 public:
  Action* inner;
  explicit RecAction(Action* a) : inner(a) {}
  virtual double getActionDifference(const SectionSamplerInterface& s, int level) {
    double d = inner->getActionDifference(s, level);
    if (g_rec) {
      g_rec->ds[level] = d;
      g_rec->ipart = s.getMovingIndex()(0);
    }
    return d;
  }
  virtual double getActionDifference(const Paths& p, const VArray& disp, int n,
                                     const IArray& idx, int f, int l) {
    const double d = inner->getActionDifference(p, disp, n, idx, f, l);
    if (g_drec) g_drec->ds += d;
    return d;
  }
  virtual double getTotalAction(const Paths& p, const int level) const {
    return inner->getTotalAction(p, level);
  }
  virtual void getBeadAction(const Paths& p, int ipart, int islice, double& u,
                             double& utau, double& ulambda, Vec& fm, Vec& fp) const {
    inner->getBeadAction(p, ipart, islice, u, utau, ulambda, fm, fp);
  }
  virtual void initialize(const SectionChooser& c) { inner->initialize(c); }
  virtual void acceptLastMove() {
    inner->acceptLastMove();
    g_accepted = true;
  }
};

class RecDoubleAction : public DoubleAction {
 public:
  DoubleAction* inner;
  explicit RecDoubleAction(DoubleAction* a) : inner(a) {}
  virtual double getActionDifference(const SectionSamplerInterface& s, const int level) {
    double d = inner->getActionDifference(s, level);
    if (g_rec) g_rec->ds_node[level] = d;
    return d;
  }
  virtual double getActionDifference(const Paths& p, const VArray& disp, int n,
                                     const IArray& idx, int f, int l) {
    const double d = inner->getActionDifference(p, disp, n, idx, f, l);
    if (g_drec) g_drec->ds_node += d;
    return d;
  }
  virtual double getTotalAction(const Paths& p, const int level) const {
    return inner->getTotalAction(p, level);
  }
  virtual void getBeadAction(const Paths& p, int ipart, int islice, double& u,
                             double& utau, double& ulambda, Vec& fm, Vec& fp) const {
    inner->getBeadAction(p, ipart, islice, u, utau, ulambda, fm, fp);
  }
  virtual void initialize(const DoubleSectionChooser& c) { inner->initialize(c); }
  virtual void acceptLastMove() { inner->acceptLastMove(); }
};

class RecMover : public Mover {
 public:
  Mover* inner;
  explicit RecMover(Mover* m) : inner(m) {}
  virtual ~RecMover() { delete inner; }
  virtual double makeMove(MultiLevelSampler& s, const int level) {
    double v = inner->makeMove(s, level);
    if (g_rec) g_rec->lnt[level] = v;
    if (level < g_lowest_level) g_lowest_level = level;
    return v;
  }
  virtual double makeDelayedMove(MultiLevelSampler& s, const int level) {
    return inner->makeDelayedMove(s, level);
  }
  virtual double getForwardProb() { return inner->getForwardProb(); }
};

// Sums over links like ThermoEnergyEstimator::handleLink
// (src/estimator/ThermoEnergyEstimator.cc:32-50) with endCalc dividing by nslice.
class ThermoSum : public LinkSummable {
 public:
  const Action* action;
  const DoubleAction* daction;
  double sum;
  ThermoSum(const Action* a, const DoubleAction* d) : action(a), daction(d), sum(0) {}
  virtual void initCalc(const int, const int) { sum = 0; }
  virtual void handleLink(const Vec&, const Vec&, int ipart, int islice, const Paths& paths) {
    double u = 0, utau = 0, ul = 0;
    Vec fm, fp;
    if (action) {
      action->getBeadAction(paths, ipart, islice, u, utau, ul, fm, fp);
      sum += utau;
    }
    if (daction) {
      u = 0; utau = 0; ul = 0;
      daction->getBeadAction(paths, ipart, islice, u, utau, ul, fm, fp);
      sum += utau;
    }
  }
};

// A fixed section/moving-bead pair for Action-level calls, like
// unit-tests/advancer/MultiLevelSamplerFake.
class FakeSampler : public SectionSamplerInterface {
 public:
  Beads<NDIM>* section;
  Beads<NDIM>* moving;
  IArray index;
  const SuperCell* cell;
  FakeSampler(int npart, int nmoving, int nslice, const SuperCell* c)
      : section(new Beads<NDIM>(npart, nslice)),
        moving(new Beads<NDIM>(nmoving, nslice)),
        index(nmoving),
        cell(c) {}
  ~FakeSampler() {
    delete section;
    delete moving;
  }
  virtual const Beads<NDIM>& getSectionBeads() const { return *section; }
  virtual const Beads<NDIM>& getSectionBeads(int) const { return *section; }
  virtual const Beads<NDIM>& getMovingBeads() const { return *moving; }
  virtual const Beads<NDIM>& getMovingBeads(int) const { return *moving; }
  virtual Beads<NDIM>& getSectionBeads() { return *section; }
  virtual Beads<NDIM>& getSectionBeads(int) { return *section; }
  virtual Beads<NDIM>& getMovingBeads() { return *moving; }
  virtual Beads<NDIM>& getMovingBeads(int) { return *moving; }
  virtual const IArray& getMovingIndex() const { return index; }
  virtual const IArray& getMovingIndex(int) const { return index; }
  virtual int getFirstSliceIndex() const { return 0; }
  virtual const SuperCell& getSuperCell() const { return *cell; }
  virtual bool isSamplingBoth() const { return false; }
};

// ---- the simulation object -----------------------------------------------
struct RefSim {
  ora_config cfg;
  SimulationInfo* simInfo;
  SerialPaths* paths;
  CompositeAction* composite;
  CoulombAction* coulomb;
  CompositeDoubleAction* dcomposite;
  std::vector<NodeModel*> nodes;  // per species (0 when none)
  RecAction* rec;
  RecDoubleAction* drec;
  RecMover* mover;
  SectionChooser* chooser;
  DoubleSectionChooser* dchooser;
  uint32_t next_attempt;
};

extern "C" void* ref_create(const ora_config* c) {
  RefSim* s = new RefSim();
  s->cfg = *c;
  const int nspec = c->nspecies;
  SuperCell* cell = new SuperCell(Vec(c->cell[0], c->cell[1], c->cell[2]));
  std::vector<Species*> specList(nspec), specIndex(c->npart);
  static const char* names[ORA_MAX_SPECIES] = {"up", "dn", "s2", "s3"};
  int ifirst = 0;
  for (int i = 0; i < nspec; ++i) {
    Species* sp = new Species(names[i], c->spec_count[i], c->spec_mass[i],
                              c->spec_charge[i], 1, true);
    sp->ifirst = ifirst;
    sp->isStatic = false;
    sp->displace = 0;
    for (int k = 0; k < c->spec_count[i]; ++k) specIndex[ifirst + k] = sp;
    ifirst += c->spec_count[i];
    specList[i] = sp;
  }
  s->simInfo = new SimulationInfo(cell, c->npart, specList, specIndex, c->temperature,
                                  c->tau, c->nslice);
  SimulationInfo& si = *s->simInfo;
  BeadFactory& bf = si.getBeadFactory();
  s->paths = new SerialPaths(c->npart, c->nslice, c->tau, *cell, bf);

  s->composite = new CompositeAction(0);
  if (c->spring) s->composite->addAction(new SpringAction(si, c->nlevel, 0.02));
  for (int i = 0; i < nspec; ++i) {
    if (c->sho_omega[i] > 0)
      s->composite->addAction(new SHOAction(c->tau, c->sho_omega[i], c->spec_mass[i],
                                            NDIM, si.getSpecies(i), Vec(0.0)));
    if (c->prim_a[i] != 0 || c->prim_b[i] != 0)
      s->composite->addAction(
          new PrimSHOAction(c->prim_a[i], c->prim_b[i], si, NDIM, si.getSpecies(i)));
  }
  s->coulomb = 0;
  if (c->coulomb) {
    s->coulomb = new CoulombAction(c->epsilon, si, c->norder, 0.0, 0.0, c->ngpts, false,
                                   c->ewald != 0, NDIM, c->ewald_rcut, c->ewald_kcut, 0.0,
                                   0.0, 1, "optEwald", 0);
    s->composite->addAction(s->coulomb);
  }
  s->rec = new RecAction(s->composite);

  bool fixedNode = false;
  s->nodes.assign(nspec, (NodeModel*)0);
  s->dcomposite = new CompositeDoubleAction(0);
  for (int i = 0; i < nspec; ++i) {
    NodeModel* nm = 0;
    if (c->node_kind[i] == 1) {
      nm = new SHONodes(si, si.getSpecies(i), c->node_omega[i], c->node_temperature,
                        c->nlevel);
    } else if (c->node_kind[i] == 2) {
      nm = new FreeParticleNodes(si, si.getSpecies(i), c->node_temperature, c->nlevel,
                                 false, 0, false, 0, 5.0);
    }
    if (nm) {
      fixedNode = true;
      s->nodes[i] = nm;
      s->dcomposite->addAction(new FixedNodeAction(si, si.getSpecies(i), nm, true, false,
                                                   c->nlevel, false, 1000, 0));
    }
  }
  s->drec = fixedNode ? new RecDoubleAction(s->dcomposite) : 0;

  Mover* inner = (c->mover == 1) ? (Mover*)new FreeMoverPBC(si, c->nlevel, 10.0)
                                 : (Mover*)new FreeMover(si, c->nlevel, 10.0);
  s->mover = new RecMover(inner);
  s->chooser = 0;
  s->dchooser = 0;
  // <Sample delayedRejection defaultSigmaFactor newSigmaFactor>, defaulted as
  // PIMCParser does (src/parser/PIMCParser.cc:312-322)
  const bool dr = c->delayed_rejection != 0;
  const double defaultFactor = c->sigma_factor != 0 ? c->sigma_factor : 1.0;
  const double newFactor = (dr && c->dr_sigma_factor == 0) ? 0.75 : c->dr_sigma_factor;
  if (!fixedNode) {
    s->chooser = new SectionChooser(c->nlevel, c->npart, *s->paths, *s->rec, bf);
    MultiLevelSampler* ml = new MultiLevelSampler(
        1, *s->paths, *s->chooser, new SimpleParticleChooser(c->npart, 1),
        new PermutationChooser(1), *s->mover, s->rec, 1, bf, dr, defaultFactor, newFactor,
        true);
    s->chooser->resize(1);
    s->chooser->set(0, ml);
  } else {
    s->dchooser =
        new DoubleSectionChooser(c->nlevel, c->npart, *s->paths, *s->rec, *s->drec, bf);
    DoubleMLSampler* ml = new DoubleMLSampler(
        1, *s->paths, *s->dchooser, new SimpleParticleChooser(c->npart, 1),
        new PermutationChooser(1), new SimpleParticleChooser(c->npart, 1), 0, *s->mover,
        s->rec, s->drec, false, 1, bf, dr, defaultFactor, newFactor, true);
    s->dchooser->resize(1);
    s->dchooser->set(0, ml);
  }
  s->next_attempt = 0;
  return s;
}

// Hooks for the pi-qmc-side adapters test: the composite action, or one
// species' node model inside its FixedNodeAction, replaced by another object of
// the same pi-qmc interface, so that pi-qmc's own samplers, section choosers
// and FixedNodeAction run on it.  `action` is an Action*, `model` a NodeModel*.
extern "C" void ref_replace_action(void* h, void* action) {
  RefSim* s = (RefSim*)h;
  s->rec->inner = (Action*)action;
}

extern "C" int ref_replace_node_model(void* h, int ispec, void* model) {
  RefSim* s = (RefSim*)h;
  if (!s->dcomposite || ispec < 0 || ispec >= (int)s->nodes.size() || !s->nodes[ispec]) return -1;
  int first = 0;
  for (int i = 0; i < ispec; ++i) first += s->cfg.spec_count[i];
  for (size_t k = 0; k < s->dcomposite->actions.size(); ++k) {
    FixedNodeAction* f = dynamic_cast<FixedNodeAction*>(s->dcomposite->actions[k]);
    if (f && f->ifirst == first) {
      f->nodeModel = (NodeModel*)model;
      f->matrixUpdateObj = 0;
      s->nodes[ispec] = (NodeModel*)model;
      return 0;
    }
  }
  return -1;
}

// The SerialPaths object (a Paths&) and the SimulationInfo of a simulation,
// for adapters that take them.
extern "C" void* ref_paths(void* h) { return (Paths*)((RefSim*)h)->paths; }
extern "C" void* ref_simulation_info(void* h) { return ((RefSim*)h)->simInfo; }

extern "C" void ref_destroy(void* h) {
  // The reference objects hold cross references without clear ownership; the
  // checker process is short-lived, so they are left for process exit.
  (void)h;
}

extern "C" void ref_set_path(void* h, const double* xyz) {
  RefSim* s = (RefSim*)h;
  const int np = s->cfg.npart, ns = s->cfg.nslice;
  for (int t = 0; t < ns; ++t)
    for (int i = 0; i < np; ++i)
      for (int d = 0; d < 3; ++d) (*s->paths)(i, t)[d] = xyz[(t * np + i) * 3 + d];
}

extern "C" void ref_get_path(void* h, double* xyz) {
  RefSim* s = (RefSim*)h;
  const int np = s->cfg.npart, ns = s->cfg.nslice;
  for (int t = 0; t < ns; ++t)
    for (int i = 0; i < np; ++i)
      for (int d = 0; d < 3; ++d) xyz[(t * np + i) * 3 + d] = (*s->paths)(i, t)[d];
}

// WritePaths::run (src/algorithm/WritePaths.cc:25-114) on the current path:
// dumpFreq 0 writes on the first call; no movie file.
extern "C" void ref_write_paths(void* h, const char* filename) {
  RefSim* s = (RefSim*)h;
  WritePaths w(*s->paths, std::string(filename), 0, 1, false, *s->simInfo, 0,
               s->simInfo->getBeadFactory());
  w.run();
}

// PathReader::run (src/algorithm/PathReader.cc:20-140) into the current path.
extern "C" void ref_read_paths(void* h, const char* filename, int bfactor) {
  RefSim* s = (RefSim*)h;
  std::string name(filename);
  PathReader r(*s->paths, name, s->simInfo->getBeadFactory(), bfactor, 0);
  r.run();
}

// Runs n section-move attempts numbered first_attempt, first_attempt+1, ...
// Returns the number accepted.
extern "C" int ref_run(void* h, int n, uint32_t first_attempt, ora_record* recs) {
  RefSim* s = (RefSim*)h;
  int nacc = 0;
  for (int a = 0; a < n; ++a) {
    ora_record dummy;
    ora_record* r = recs ? &recs[a] : &dummy;
    for (int l = 0; l <= ORA_MAX_LEVEL; ++l) r->ds[l] = r->ds_node[l] = r->lnt[l] = 0;
    r->ipart = -1;
    g_rec = r;
    g_accepted = false;
    g_lowest_level = 99;
    shim_begin_attempt(s->cfg.seed, s->cfg.replica, first_attempt + (uint32_t)a);
    if (s->chooser) {
      s->chooser->run();
      r->ifirst1 = s->chooser->iFirstSlice;
      r->ifirst2 = -2;
    } else {
      s->dchooser->run();
      r->ifirst1 = s->dchooser->iFirstSlice1;
      r->ifirst2 = s->dchooser->iFirstSlice2;
    }
    r->reject_level = g_accepted ? -1 : g_lowest_level;
    if (g_accepted) ++nacc;
    g_rec = 0;
  }
  return nacc;
}

// Runs n rigid-displacement attempts (DisplaceMoveSampler::run with nrepeat 1,
// src/advancer/DisplaceMoveSampler.cc:63-224; DoubleDisplaceMoveSampler for
// fixed-node systems, src/advancer/DoubleDisplaceMoveSampler.cc:40-128) with a
// UniformMover of box dist and a SimpleParticleChooser (species < 0) or a
// SpeciesParticleChooser.  Returns the number accepted.
extern "C" int ref_run_displace(void* h, int n, uint32_t first_attempt, const double* dist,
                                int nmoving, int species, ora_drecord* recs) {
  RefSim* s = (RefSim*)h;
  UniformMover mover(Vec(dist[0], dist[1], dist[2]), 0);
  ParticleChooser* pc =
      species < 0 ? (ParticleChooser*)new SimpleParticleChooser(s->cfg.npart, nmoving)
                  : (ParticleChooser*)new SpeciesParticleChooser(s->simInfo->getSpecies(species),
                                                                 nmoving);
  DisplaceMoveSampler* smp =
      s->drec ? (DisplaceMoveSampler*)new DoubleDisplaceMoveSampler(
                    nmoving, 1, *s->paths, *pc, mover, s->rec, s->drec, 0)
              : new DisplaceMoveSampler(nmoving, 1, *s->paths, *pc, mover, s->rec, 0);
  smp->getAccRejEstimator("displace");
  int nacc = 0;
  for (int a = 0; a < n; ++a) {
    ora_drecord dummy;
    ora_drecord* r = recs ? &recs[a] : &dummy;
    memset(r, 0, sizeof(*r));
    g_drec = r;
    g_accepted = false;
    shim_begin_attempt(s->cfg.seed, s->cfg.replica, first_attempt + (uint32_t)a);
    smp->run();
    for (int i = 0; i < nmoving && i < ORA_MAX_MOVING; ++i) {
      r->ipart[i] = smp->movingIndex(i);
      for (int d = 0; d < 3; ++d) r->disp[i][d] = smp->displacement(i)[d];
    }
    r->accepted = g_accepted ? 1 : 0;
    if (g_accepted) ++nacc;
    g_drec = 0;
  }
  return nacc;
}

// pi-qmc's own estimators over the current paths (one evaluate() each):
// VirialEnergyEstimator (src/estimator/VirialEnergyEstimator.cc:34-79) over the
// composite and double actions, CoulombEnergyEstimator
// (src/estimator/CoulombEnergyEstimator.cc:30-44) and the optimized-Ewald
// EwaldCoulombEstimator (src/estimator/EwaldCoulombEstimator.cc:60-140).
extern "C" double ref_virial_energy(void* h, int nwindow) {
  RefSim* s = (RefSim*)h;
  VirialEnergyEstimator est(*s->simInfo, s->composite, s->drec ? s->dcomposite : 0, nwindow, 0,
                            "", 1.0, 0.0);
  est.evaluate(*s->paths);
  return est.calcValue();
}

extern "C" double ref_coulomb_energy(void* h, double epsilon) {
  RefSim* s = (RefSim*)h;
  SimpleScalarAccumulator* acc = new SimpleScalarAccumulator(0);
  CoulombEnergyEstimator est(*s->simInfo, epsilon, "", 1.0, 0.0, acc);
  est.evaluate(*s->paths);
  return acc->getValue();
}

extern "C" double ref_ewald_coulomb_energy(void* h, double epsilon, double rcut, double kcut) {
  RefSim* s = (RefSim*)h;
  SimpleScalarAccumulator* acc = new SimpleScalarAccumulator(0);
  EwaldCoulombEstimator est(*s->simInfo, s->composite, epsilon, rcut, kcut, "", 1.0, 0.0, acc);
  est.evaluate(*s->paths);
  return acc->getValue();
}

extern "C" double ref_thermo_energy(void* h) {
  RefSim* s = (RefSim*)h;
  ThermoSum ts(s->composite, s->drec ? s->dcomposite : 0);
  s->paths->sumOverLinks(ts);
  return ts.sum / s->cfg.nslice;
}

// Per-bead action and tau-derivative (CompositeAction::getBeadAction).
extern "C" void ref_bead_action(void* h, int ipart, int islice, double* u, double* utau) {
  RefSim* s = (RefSim*)h;
  double ul = 0;
  Vec fm, fp;
  s->composite->getBeadAction(*s->paths, ipart, islice, *u, *utau, ul, fm, fp);
}

// Action-level difference of the composite Action for a given section and
// moving beads (one moving particle set), at one level.
extern "C" double ref_action_diff(void* h, int level, const double* section,
                                  const double* moving, int nmoving, const int* index) {
  RefSim* s = (RefSim*)h;
  const int np = s->cfg.npart, nsl = (1 << s->cfg.nlevel) + 1;
  FakeSampler fs(np, nmoving, nsl, s->simInfo->getSuperCell());
  for (int t = 0; t < nsl; ++t) {
    for (int i = 0; i < np; ++i)
      for (int d = 0; d < 3; ++d) (*fs.section)(i, t)[d] = section[(t * np + i) * 3 + d];
    for (int m = 0; m < nmoving; ++m)
      for (int d = 0; d < 3; ++d) (*fs.moving)(m, t)[d] = moving[(t * nmoving + m) * 3 + d];
  }
  for (int m = 0; m < nmoving; ++m) fs.index(m) = index[m];
  return s->composite->getActionDifference(fs, level);
}

// NodeModel::evaluate + evaluateDistance for one species on slice-cache islice.
extern "C" int ref_node_eval(void* h, int ispec, const double* r1, const double* r2,
                             int islice, int scale_magnitude, double* det, double* d1,
                             double* d2) {
  RefSim* s = (RefSim*)h;
  NodeModel* nm = s->nodes[ispec];
  if (!nm) return -1;
  const int np = s->cfg.npart;
  NodeModel::VArray a1(np), a2(np);
  for (int i = 0; i < np; ++i)
    for (int d = 0; d < 3; ++d) {
      a1(i)[d] = r1[i * 3 + d];
      a2(i)[d] = r2[i * 3 + d];
    }
  NodeModel::DetWithFlag res = nm->evaluate(a1, a2, islice, scale_magnitude != 0);
  *det = res.det;
  NodeModel::Array b1(np), b2(np);
  nm->evaluateDistance(a1, a2, islice, b1, b2);
  for (int i = 0; i < np; ++i) {
    d1[i] = b1(i);
    d2[i] = b2(i);
  }
  return res.err ? 1 : 0;
}

extern "C" double ref_node_scale(void* h, int ispec) {
  RefSim* s = (RefSim*)h;
  NodeModel* nm = s->nodes[ispec];
  if (SHONodes* sn = dynamic_cast<SHONodes*>(nm)) return sn->scale;
  if (FreeParticleNodes* fn = dynamic_cast<FreeParticleNodes*>(nm)) return fn->scale;
  return 0;
}

extern "C" void ref_set_node_scale(void* h, int ispec, double scale) {
  RefSim* s = (RefSim*)h;
  NodeModel* nm = s->nodes[ispec];
  if (SHONodes* sn = dynamic_cast<SHONodes*>(nm)) sn->scale = scale;
  if (FreeParticleNodes* fn = dynamic_cast<FreeParticleNodes*>(nm)) fn->scale = scale;
}

// Pair-action tables of the CoulombAction, in construction order.
extern "C" int ref_num_pair_tables(void* h) {
  RefSim* s = (RefSim*)h;
  return s->coulomb ? (int)s->coulomb->pairActionArray.size() : 0;
}

extern "C" int ref_pair_table(void* h, int k, int* info, double* grid_params,
                              double* ugrid) {
  RefSim* s = (RefSim*)h;
  if (!s->coulomb || k >= (int)s->coulomb->pairActionArray.size()) return -1;
  PairAction* pa = s->coulomb->pairActionArray[k];
  const int ndata = pa->ugrid.extent(2);
  info[0] = pa->ngpts;
  info[1] = pa->norder;
  info[2] = pa->ifirst1;
  info[3] = pa->npart1;
  info[4] = pa->ifirst2;
  info[5] = pa->npart2;
  info[6] = ndata;
  info[7] = pa->exLevel;
  grid_params[0] = pa->rgridinv;
  grid_params[1] = pa->logrratioinv;
  grid_params[2] = pa->mass;
  if (ugrid)
    for (int i = 0; i < pa->ngpts; ++i)
      for (int t = 0; t < 2; ++t)
        for (int kk = 0; kk < ndata; ++kk)
          ugrid[(i * 2 + t) * ndata + kk] = pa->ugrid(i, t, kk);
  return 0;
}

extern "C" int ref_ewald(void* h, int* totk, int* kvec, double* vk, double* scal,
                         int* ikmax) {
  RefSim* s = (RefSim*)h;
  if (!s->coulomb || !s->coulomb->ewaldSum) return -1;
  EwaldSum* e = s->coulomb->ewaldSum;
  *totk = e->totk;
  if (kvec)
    for (int i = 0; i < e->totk; ++i) {
      kvec[3 * i] = e->kvec(i)[0];
      kvec[3 * i + 1] = e->kvec(i)[1];
      kvec[3 * i + 2] = e->kvec(i)[2];
      vk[i] = e->vk(i);
    }
  scal[0] = e->oneOver2V;
  scal[1] = e->selfEnergy;
  if (OptEwaldSum* oe = dynamic_cast<OptEwaldSum*>(e)) {
    for (int i = 0; i < oe->npoly; ++i) scal[2 + i] = oe->coef(i);
  }
  for (int d = 0; d < 3; ++d) ikmax[d] = e->ikmax[d];
  return 0;
}

// The optimized Ewald sum an EwaldCoulombEstimator builds for itself
// (src/estimator/EwaldCoulombEstimator.cc:60-90): its k-list, v_k, 1/(2V), self
// energy and the 1001-point short-range grid vgrid(i) = -evalFR(i rcut/1000)/eps.
extern "C" int ref_estimator_ewald(void* h, double rcut, double kcut, double epsilon, int* totk,
                                   int* kvec, double* vk, double* scal, int* ikmax,
                                   double* vgrid) {
  RefSim* s = (RefSim*)h;
  const int np = s->cfg.npart;
  OptEwaldSum e(*s->simInfo->getSuperCell(), np, rcut, kcut, 4 * kcut, 8);
  for (int i = 0; i < np; ++i) e.getQArray()(i) = s->simInfo->getPartSpecies(i).charge;
  e.evalSelfEnergy();
  *totk = e.totk;
  if (kvec)
    for (int i = 0; i < e.totk; ++i) {
      kvec[3 * i] = e.kvec(i)[0];
      kvec[3 * i + 1] = e.kvec(i)[1];
      kvec[3 * i + 2] = e.kvec(i)[2];
      vk[i] = e.vk(i);
    }
  scal[0] = e.oneOver2V;
  scal[1] = e.selfEnergy;
  for (int d = 0; d < 3; ++d) ikmax[d] = e.ikmax[d];
  if (vgrid) {
    const double dr = rcut / 1000;
    vgrid[0] = -e.evalFR0() / epsilon;
    for (int i = 1; i < 1001; ++i) vgrid[i] = -e.evalFR(i * dr) / epsilon;
  }
  return 0;
}

extern "C" double ref_ewald_long_range(void* h, const double* r) {
  RefSim* s = (RefSim*)h;
  EwaldSum* e = s->coulomb->ewaldSum;
  const int np = s->cfg.npart;
  EwaldSum::VArray rv(np);
  for (int i = 0; i < np; ++i) rv(i) = Vec(r[3 * i], r[3 * i + 1], r[3 * i + 2]);
  return e->evalLongRange(rv);
}

// Pair potential helpers: CoulombAction::u / utau (last pair's mu, q1q2).
extern "C" double ref_coulomb_u(void* h, double r, int order) {
  RefSim* s = (RefSim*)h;
  return s->coulomb->u(r, order);
}
extern "C" double ref_coulomb_utau(void* h, double r, int order) {
  RefSim* s = (RefSim*)h;
  return s->coulomb->utau(r, order);
}
