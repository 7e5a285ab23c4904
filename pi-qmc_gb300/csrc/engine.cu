// Host side of the engine: the C ABI declared in include/pimc_gb300.h.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/pimc_gb300.h"
#include "kernels.cuh"

using namespace pimc;

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

#define CU(call)                                                                      \
  do {                                                                                \
    cudaError_t e_ = (call);                                                          \
    if (e_ != cudaSuccess)                                                            \
      return fail(PIMC_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

template <class T>
struct DevBuf {
  T* p = nullptr;
  size_t n = 0;
  int alloc(size_t count) {
    free();
    n = count;
    if (count == 0) return 0;
    if (cudaMalloc(&p, count * sizeof(T)) != cudaSuccess) {
      p = nullptr;
      return -1;
    }
    return 0;
  }
  void free() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
};

}  // namespace

struct pimc_engine {
  int nrep = 0;
  int precision = PIMC_PREC_FP64;
  uint64_t seed = 0;
  cudaStream_t stream = nullptr;
  std::vector<DevSys> hsys;
  std::vector<pimc_system> hdesc;
  std::vector<long long> path_off;  // nrep+1
  DevBuf<DevSys> d_sys;
  DevBuf<DevState> d_state;
  DevBuf<double> d_paths;
  DevBuf<double> d_nodescr;
  DevBuf<double> d_nodecache;
  DevBuf<int> d_order;
  DevBuf<int> d_next;
  DevBuf<double> d_ugrid;
  DevBuf<float> d_ugrid32;
  DevBuf<int> d_kvec;
  DevBuf<double> d_vk;
  Layout lay{};
  int block = kBlock;
  int grid = 0;
  int num_sms = 0;
  long long launches = 0;
  ~pimc_engine() {
    d_sys.free();
    d_state.free();
    d_paths.free();
    d_nodescr.free();
    d_nodecache.free();
    d_order.free();
    d_next.free();
    d_ugrid.free();
    d_ugrid32.free();
    d_kvec.free();
    d_vk.free();
  }
};

namespace {

// PeriodicGaussian constructor constants (src/util/PeriodicGaussian.cc:7-18).
void pg_params(double alpha, double length, double& nome, double& pref, double& k, int& nmax) {
  const double PI = 3.141592653589793;
  nome = std::exp(-PI * PI / (alpha * length * length));
  nmax = 1 + int(2.0 * std::sqrt(alpha * length * length));
  pref = std::sqrt(PI / (alpha * length * length));
  k = 2 * PI / length;
}

int validate(const pimc_system& s) {
  if (s.npart <= 0 || s.nspecies <= 0 || s.nspecies > PIMC_MAX_SPECIES)
    return fail(PIMC_ERR_INVALID, "npart/nspecies out of range");
  int tot = 0;
  for (int i = 0; i < s.nspecies; ++i) {
    if (s.spec_count[i] <= 0 || !(s.spec_mass[i] > 0))
      return fail(PIMC_ERR_INVALID, "species count and mass must be positive");
    tot += s.spec_count[i];
    if (s.node_kind[i] && s.spec_count[i] > PIMC_MAX_NODE_PARTICLES)
      return fail(PIMC_ERR_CAPACITY, "node-model species larger than 32 particles");
  }
  if (tot != s.npart) return fail(PIMC_ERR_INVALID, "species counts do not add up to npart");
  if (s.nlevel < 1 || s.nlevel > PIMC_MAX_LEVEL)
    return fail(PIMC_ERR_CAPACITY, "nlevel must be in 1..6");
  if (s.nslice < (1 << s.nlevel) + 1) return fail(PIMC_ERR_INVALID, "nslice smaller than a section");
  if (!(s.tau > 0)) return fail(PIMC_ERR_INVALID, "tau must be positive");
  bool fixed = false;
  for (int i = 0; i < s.nspecies; ++i) fixed |= s.node_kind[i] != 0;
  if (fixed && (s.nslice % 2)) return fail(PIMC_ERR_INVALID, "fixed node needs an even nslice");
  if (fixed && !(s.node_temperature > 0))
    return fail(PIMC_ERR_INVALID, "fixed node needs node_temperature > 0");
  // Periodic-Gaussian springs/movers (boxes smaller than the bisection width)
  // are outside this engine's scope.
  for (int i = 0; i < s.nspecies; ++i)
    for (int lev = 0; lev <= s.nlevel + 1; ++lev)
      for (int d = 0; d < 3; ++d) {
        const double L = s.cell[d];
        const double am = s.spec_mass[i] / (s.tau * (1 << lev));
        const double as = s.spec_mass[i] / (2 * s.tau * (1 << std::min(lev, s.nlevel)));
        if (1 + int(2.0 * std::sqrt(am * L * L)) < 16 || 1 + int(2.0 * std::sqrt(as * L * L)) < 16)
          return fail(PIMC_ERR_INVALID,
                      "cell too small: periodic-Gaussian spring/mover images are not supported");
      }
  return 0;
}

void fill_sys(const pimc_system& s, DevSys& d) {
  memset(&d, 0, sizeof(d));
  d.npart = s.npart;
  d.nspecies = s.nspecies;
  d.nslice = s.nslice;
  d.nlevel = s.nlevel;
  d.nsec = (1 << s.nlevel) + 1;
  int first = 0;
  d.ns_max = 1;
  for (int i = 0; i < s.nspecies; ++i) {
    d.spec_first[i] = first;
    d.spec_count[i] = s.spec_count[i];
    first += s.spec_count[i];
    d.mass[i] = s.spec_mass[i];
    d.lambda[i] = 0.5 / s.spec_mass[i];
    d.charge[i] = s.spec_charge[i];
    d.sho_omega[i] = s.sho_omega[i];
    d.prim_a[i] = s.prim_a[i];
    d.prim_b[i] = s.prim_b[i];
    d.node_kind[i] = s.node_kind[i];
    if (s.node_kind[i]) {
      d.fixed_node = 1;
      d.ns_max = std::max(d.ns_max, s.spec_count[i]);
    }
    if (s.node_kind[i] == PIMC_NODES_SHO) {
      // SHONodes constructor (src/fixednode/SHONodes.cc:22-29).
      const double T = s.node_temperature, w = s.node_omega[i];
      d.node_cosh[i] = std::cosh(w * 0.5 / T);
      const double sinhwt = std::sinh(w * 0.5 / T);
      d.node_c[i] = s.spec_mass[i] * 0.5 * w / sinhwt;
    } else if (s.node_kind[i] == PIMC_NODES_FREE) {
      for (int a = 0; a < 3; ++a)
        pg_params(s.spec_mass[i] * s.node_temperature, s.cell[a], d.pg_nome[i][a], d.pg_pref[i][a],
                  d.pg_k[i][a], d.pg_nmax[i][a]);
    }
  }
  d.tau = s.tau;
  for (int lev = 0; lev < kMaxLevels; ++lev) {
    const int nStride = 1 << lev;
    d.sho_div2[lev] = 1.0 / (2.0 * s.tau * nStride);
    for (int i = 0; i < s.nspecies; ++i) {
      const double lam = 0.5 / s.spec_mass[i];
      d.spr_inv2s2[lev][i] = 0.25 / (lam * s.tau * nStride);
      const double sigma = 1.0 * std::sqrt(lam * s.tau * nStride);
      d.mov_sigma[lev][i] = sigma;
      d.mov_inv2s2[lev][i] = 0.5 / (sigma * sigma);
      if (s.sho_omega[i] > 0) {
        const double wt = s.sho_omega[i] * s.tau * nStride;
        d.sho_cosh[lev][i] = std::cosh(wt);
        d.sho_div1[lev][i] = 1.0 / (2.0 * std::sinh(wt));
      }
    }
  }
  for (int i = 0; i < s.nspecies; ++i) {
    if (s.sho_omega[i] > 0) {
      const double wt = s.sho_omega[i] * s.tau;
      const double sinhwt = std::sinh(wt), coshwt = std::cosh(wt);
      d.sho_cosh0[i] = coshwt;
      d.sho_csch[i] = 1.0 / sinhwt;
      d.sho_coth[i] = coshwt * d.sho_csch[i];
    }
  }
  for (int a = 0; a < 3; ++a) {
    d.cell[a] = s.cell[a];
    d.cellb[a] = 1. / s.cell[a];
  }
  double l2 = d.cell[0] * d.cell[0];
  d.rcut2 = l2;
  for (int a = 1; a < 3; ++a) {
    l2 = d.cell[a] * d.cell[a];
    d.rcut2 = (d.rcut2 > l2) ? l2 : d.rcut2;
  }
  d.rcut2 *= 0.25;
  d.spring = s.spring;
  d.coulomb = s.coulomb;
  d.ewald = s.ewald;
  d.mover = s.mover;
  d.epsilon = s.epsilon > 0 ? s.epsilon : 1.0;
}

Layout make_layout(const std::vector<DevSys>& sys, int nwarps, bool& ok) {
  int nsec = 0, np = 0, nsm = 1, ewt = 0;
  bool fixed = false;
  for (const DevSys& d : sys) {
    nsec = std::max(nsec, d.nsec);
    np = std::max(np, d.npart);
    nsm = std::max(nsm, d.ns_max);
    fixed |= d.fixed_node != 0;
    if (d.ewald) ewt = std::max(ewt, 2 * (d.ikmax[0] + 1 + 2 * d.ikmax[1] + 1 + 2 * d.ikmax[2] + 1) * (d.npart + 1));
  }
  Layout L{};
  int off = 0;
  auto take = [&](int n) {
    const int o = off;
    off += (n + 1) & ~1;  // keep 16-byte alignment
    return o;
  };
  L.s1 = take(3 * nsec * np);
  L.s2 = take(fixed ? 3 * nsec * np : 0);
  L.mv = take(3 * nsec);
  L.red = take(64);
  L.q = take(np);
  L.dm = take(kMaxSpecies * nsec);
  L.ndm = take(nsec);
  L.edet = take(nsec);
  L.dist = take(fixed ? nsec * 2 * nsm : 0);
  L.ndist = take(fixed ? nsec * 2 * nsm : 0);
  L.ewt = take(ewt);
  L.ictl = take((C_NCTL + 2 * nsec + 1) / 2 + 1);
  bool sho = false;
  for (const DevSys& d : sys)
    for (int i = 0; i < d.nspecies; ++i) sho |= d.node_kind[i] == PIMC_NODES_SHO;
  // exp-matrix cache of the moving species' section slices; left out (the
  // levels then recompute whole matrices) when it would not fit
  L.ecache = (sho && (off + nsec * nsm * nsm) * 8 <= 120 * 1024) ? take(nsec * nsm * nsm) : -1;
  L.ncol = fixed ? take(nsec * nsm) : -1;
  // per-warp Slater scratch: (32 / W) lane groups of node_group_scratch(n) doubles
  int stride = 0;
  if (fixed)
    for (int n = 1; n <= nsm; ++n)
      stride = std::max(stride, (32 / node_group_width(n)) * node_group_scratch(n));
  L.nodescr_stride = (stride + 1) & ~1;
  const int need = off + nwarps * L.nodescr_stride;
  const int limit = 200 * 1024 / 8;
  if (need <= limit) {
    L.nodescr = take(nwarps * L.nodescr_stride);
    L.nodescr_in_smem = 1;
  } else {
    L.nodescr = -1;
    L.nodescr_in_smem = 0;
  }
  L.total = off;
  ok = L.total <= limit;
  return L;
}

int device_check(int& nsm) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return fail(PIMC_ERR_NO_DEVICE, "no CUDA device");
  cudaDeviceProp p;
  CU(cudaGetDeviceProperties(&p, dev));
  if (p.major * 10 + p.minor < 100)
    return fail(PIMC_ERR_NO_DEVICE, "device is not Blackwell-class (sm_103a build)");
  nsm = p.multiProcessorCount;
  return 0;
}

int build_engine(const pimc_system* sys, int nrep, const pimc_pair_table* tables,
                 const int* tab_off, int uniform, const pimc_ewald_table* ewald, uint64_t seed,
                 int precision, pimc_engine** out) {
  if (!sys || nrep <= 0 || !out) return fail(PIMC_ERR_INVALID, "null argument or nreplica <= 0");
  *out = nullptr;
  int nsm = 0;
  if (int rc = device_check(nsm)) return rc;
  pimc_engine* e = new pimc_engine();
  e->nrep = nrep;
  e->seed = seed;
  e->precision = precision;
  e->num_sms = nsm;
  e->hsys.resize(nrep);
  e->hdesc.resize(nrep);
  e->path_off.resize(nrep + 1);
  // pair tables: pool the unique table objects in order of appearance
  std::vector<double> pool;
  std::vector<int> kv;
  std::vector<double> vk;
  long long off = 0;
  struct Pending {
    int rep, slot;
    size_t pool_off;
  };
  std::vector<Pending> pend;
  std::map<const double*, size_t> pooled;
  for (int r = 0; r < nrep; ++r) {
    const pimc_system& s = uniform ? sys[0] : sys[r];
    if (int rc = validate(s)) {
      delete e;
      return rc;
    }
    e->hdesc[r] = s;
    fill_sys(s, e->hsys[r]);
    DevSys& d = e->hsys[r];
    int t0 = uniform ? 0 : tab_off[r], t1 = uniform ? tab_off[0] : tab_off[r + 1];
    if (s.coulomb) {
      if (t1 - t0 > kMaxTables) {
        delete e;
        return fail(PIMC_ERR_CAPACITY, "too many pair tables");
      }
      d.ntab = 0;
      for (int k = t0; k < t1; ++k) {
        const pimc_pair_table& t = tables[k];
        if (t.species1 < 0 || t.species1 >= s.nspecies || t.species2 < 0 ||
            t.species2 >= s.nspecies || t.ngpts < 2 || t.norder < 0 || !t.ugrid) {
          delete e;
          return fail(PIMC_ERR_INVALID, "bad pair table");
        }
        DevTable& dt = d.tab[d.ntab];
        dt.ngpts = t.ngpts;
        dt.norder = t.norder;
        dt.ndata = t.norder + 1;
        dt.s1 = t.species1;
        dt.s2 = t.species2;
        dt.ifirst1 = d.spec_first[t.species1];
        dt.npart1 = d.spec_count[t.species1];
        dt.ifirst2 = d.spec_first[t.species2];
        dt.npart2 = d.spec_count[t.species2];
        dt.rgridinv = t.rgridinv;
        dt.logrratioinv = t.logrratioinv;
        // one device copy per distinct host table (replicas of a batch share them)
        size_t po = pool.size();
        auto hit = pooled.find(t.ugrid);
        if (hit != pooled.end()) {
          po = hit->second;
        } else {
          pool.insert(pool.end(), t.ugrid, t.ugrid + (size_t)t.ngpts * 2 * dt.ndata);
          pooled[t.ugrid] = po;
        }
        pend.push_back({r, d.ntab, po});
        d.ntab++;
      }
    }
    if (s.ewald) {
      if (!s.coulomb || !ewald || ewald->totk <= 0) {
        delete e;
        return fail(PIMC_ERR_INVALID, "ewald needs coulomb and an Ewald table");
      }
      d.totk = ewald->totk;
      d.one_over_2v = ewald->one_over_2v;
      d.self_energy = ewald->self_energy;
      for (int a = 0; a < 3; ++a) {
        d.ikmax[a] = ewald->ikmax[a];
        d.deltak[a] = 2 * 3.14159265358979 * d.cellb[a];
      }
    }
    d.path_offset = off;
    e->path_off[r] = off;
    off += 3LL * s.nslice * s.npart;
  }
  e->path_off[nrep] = off;
  // Block size: the widest level-0 work list decides.  Small systems without
  // node models run one or two warps per replica so that replicas pack densely.
  {
    int items = 0;
    bool fixed = false;
    for (const DevSys& d : e->hsys) {
      const int links = 1 << d.nlevel;
      items = std::max(items, links * std::max(1, d.npart));
      fixed |= d.fixed_node != 0;
    }
    e->block = fixed ? kBlock : (items <= 64 ? 64 : (items <= 128 ? 128 : kBlock));
  }
  for (DevSys& d : e->hsys) d.mixed = precision == PIMC_PREC_MIXED;
  bool ok = false;
  e->lay = make_layout(e->hsys, e->block / 32, ok);
  if (!ok) {
    delete e;
    return fail(PIMC_ERR_CAPACITY, "working set does not fit in shared memory");
  }
  // device buffers
  if (e->d_ugrid.alloc(pool.size()) || e->d_ugrid32.alloc(pool.size())) {
    delete e;
    return fail(PIMC_ERR_CUDA, "cudaMalloc pair tables");
  }
  if (!pool.empty()) {
    std::vector<float> p32(pool.begin(), pool.end());
    cudaMemcpy(e->d_ugrid.p, pool.data(), pool.size() * 8, cudaMemcpyHostToDevice);
    cudaMemcpy(e->d_ugrid32.p, p32.data(), p32.size() * 4, cudaMemcpyHostToDevice);
  }
  for (const Pending& p : pend) {
    e->hsys[p.rep].tab[p.slot].ugrid = e->d_ugrid.p + p.pool_off;
    e->hsys[p.rep].tab[p.slot].ugrid32 = e->d_ugrid32.p + p.pool_off;
  }
  if (ewald && e->hsys[0].ewald) {
    if (e->d_kvec.alloc(3 * ewald->totk) || e->d_vk.alloc(ewald->totk)) {
      delete e;
      return fail(PIMC_ERR_CUDA, "cudaMalloc Ewald table");
    }
    cudaMemcpy(e->d_kvec.p, ewald->kvec, 3 * ewald->totk * sizeof(int), cudaMemcpyHostToDevice);
    cudaMemcpy(e->d_vk.p, ewald->vk, ewald->totk * sizeof(double), cudaMemcpyHostToDevice);
    for (DevSys& d : e->hsys) {
      if (d.ewald) {
        d.kvec = e->d_kvec.p;
        d.vk = e->d_vk.p;
      }
    }
  }
  // launch geometry: persistent grid over replicas
  cudaFuncSetAttribute(section_moves_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       e->lay.total * 8);
  cudaFuncSetAttribute(thermo_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       e->lay.total * 8);
  cudaFuncSetAttribute(action_diff_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       e->lay.total * 8);
  int occ = 1;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, section_moves_kernel, e->block,
                                                e->lay.total * 8);
  occ = std::max(occ, 1);
  e->grid = std::min(nrep, nsm * occ);
  if (!e->lay.nodescr_in_smem) {
    for (DevSys& d : e->hsys) d.inv_offset = 0;
    if (e->d_nodescr.alloc((size_t)e->grid * (e->block / 32) * e->lay.nodescr_stride)) {
      delete e;
      return fail(PIMC_ERR_CUDA, "cudaMalloc node scratch");
    }
  } else {
    for (DevSys& d : e->hsys) d.inv_offset = -1;
  }
  // Slater-result cache: per replica, per species, per path slice.  Left out
  // when the two sections of an attempt can overlap (2^L >= M/2).
  {
    long long coff = 0;
    for (DevSys& d : e->hsys) {
      const bool use = d.fixed_node && (1 << d.nlevel) < d.nslice / 2;
      d.nc_stride = (2 + 2 * d.ns_max + d.ns_max * d.ns_max + 1) & ~1;
      if (use) {
        d.nc_offset = coff;
        coff += (long long)d.nspecies * d.nslice * d.nc_stride;
      } else {
        d.nc_offset = -1;
      }
    }
    if (coff > 0) {
      if (e->d_nodecache.alloc(coff)) {
        delete e;
        return fail(PIMC_ERR_CUDA, "cudaMalloc node cache");
      }
      cudaMemset(e->d_nodecache.p, 0xff, coff * sizeof(double));  // NaN epochs: all invalid
    }
  }
  if (e->d_sys.alloc(nrep) || e->d_state.alloc(nrep) || e->d_paths.alloc(off)) {
    delete e;
    return fail(PIMC_ERR_CUDA, "cudaMalloc engine state");
  }
  cudaMemcpy(e->d_sys.p, e->hsys.data(), nrep * sizeof(DevSys), cudaMemcpyHostToDevice);
  {
    // longest-processing-time-first order of the work queue
    std::vector<double> cost(nrep);
    for (int r = 0; r < nrep; ++r) {
      const DevSys& d = e->hsys[r];
      double c = (double)d.npart * d.npart;
      for (int i = 0; i < d.nspecies; ++i)
        if (d.node_kind[i]) c += 2.0 * d.spec_count[i] * d.spec_count[i] * (d.spec_count[i] + 20);
      cost[r] = c * ((1 << d.nlevel) + 1);
    }
    std::vector<int> order(nrep);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return cost[a] > cost[b]; });
    if (e->d_order.alloc(nrep) || e->d_next.alloc(1)) {
      delete e;
      return fail(PIMC_ERR_CUDA, "cudaMalloc work queue");
    }
    cudaMemcpy(e->d_order.p, order.data(), nrep * sizeof(int), cudaMemcpyHostToDevice);
  }
  std::vector<DevState> st(nrep);
  for (DevState& x : st) {
    memset(&x, 0, sizeof(x));
    for (int k = 0; k < kMaxSpecies; ++k) {
      x.node_scale[k] = 1.0;
      x.epoch[k] = 0;
    }
  }
  cudaMemcpy(e->d_state.p, st.data(), nrep * sizeof(DevState), cudaMemcpyHostToDevice);
  cudaMemset(e->d_paths.p, 0, off * sizeof(double));
  CU(cudaDeviceSynchronize());
  *out = e;
  return PIMC_OK;
}

}  // namespace

extern "C" {

const char* pimc_last_error(void) { return g_err.c_str(); }

int pimc_engine_create(const pimc_system* sys, int nreplica, const pimc_pair_table* tables,
                       int ntables, const pimc_ewald_table* ewald, uint64_t seed, int precision,
                       pimc_engine** out) {
  int toff[1] = {ntables};
  if (ntables > 0 && !tables) return fail(PIMC_ERR_INVALID, "null pair tables");
  return build_engine(sys, nreplica, tables, toff, 1, ewald, seed, precision, out);
}

int pimc_engine_create_batch(const pimc_system* sys, int nreplica, const pimc_pair_table* tables,
                             const int* table_offset, uint64_t seed, int precision,
                             pimc_engine** out) {
  if (!table_offset) return fail(PIMC_ERR_INVALID, "null table_offset");
  for (int r = 0; r < nreplica; ++r)
    if (sys[r].ewald) return fail(PIMC_ERR_INVALID, "batched engines take no Ewald systems");
  return build_engine(sys, nreplica, tables, table_offset, 0, nullptr, seed, precision, out);
}

int pimc_engine_destroy(pimc_engine* e) {
  delete e;
  return PIMC_OK;
}

int pimc_set_stream(pimc_engine* e, void* stream) {
  if (!e) return fail(PIMC_ERR_INVALID, "null engine");
  e->stream = (cudaStream_t)stream;
  return PIMC_OK;
}

int pimc_upload_paths(pimc_engine* e, const double* host_xyz) {
  if (!e || !host_xyz) return fail(PIMC_ERR_INVALID, "null argument");
  CU(cudaMemcpyAsync(e->d_paths.p, host_xyz, e->path_off[e->nrep] * sizeof(double),
                     cudaMemcpyHostToDevice, e->stream));
  if (e->d_nodecache.p)  // new paths: every cached Slater result is stale
    CU(cudaMemsetAsync(e->d_nodecache.p, 0xff, e->d_nodecache.n * sizeof(double), e->stream));
  return PIMC_OK;
}

int pimc_download_paths(pimc_engine* e, double* host_xyz) {
  if (!e || !host_xyz) return fail(PIMC_ERR_INVALID, "null argument");
  CU(cudaMemcpyAsync(host_xyz, e->d_paths.p, e->path_off[e->nrep] * sizeof(double),
                     cudaMemcpyDeviceToHost, e->stream));
  CU(cudaStreamSynchronize(e->stream));
  return PIMC_OK;
}

int pimc_path_offsets(pimc_engine* e, int64_t* offsets) {
  if (!e || !offsets) return fail(PIMC_ERR_INVALID, "null argument");
  for (int r = 0; r <= e->nrep; ++r) offsets[r] = e->path_off[r];
  return PIMC_OK;
}

int pimc_run_sections(pimc_engine* e, int nattempt, pimc_move_record* records) {
  if (!e || nattempt < 0) return fail(PIMC_ERR_INVALID, "bad argument");
  if (nattempt == 0) return PIMC_OK;
  pimc_move_record* d_rec = nullptr;
  if (records) {
    CU(cudaMallocAsync(&d_rec, sizeof(pimc_move_record) * (size_t)e->nrep * nattempt, e->stream));
    CU(cudaMemsetAsync(d_rec, 0, sizeof(pimc_move_record) * (size_t)e->nrep * nattempt, e->stream));
  }
  RunParams P;
  P.sys = e->d_sys.p;
  P.state = e->d_state.p;
  P.paths = e->d_paths.p;
  P.nodescr_g = e->d_nodescr.p;
  P.nodecache = e->d_nodecache.p;
  P.rec = d_rec;
  P.order = e->d_order.p;
  P.next = e->d_next.p;
  CU(cudaMemsetAsync(e->d_next.p, 0, sizeof(int), e->stream));
  P.nattempt = nattempt;
  P.nrep = e->nrep;
  P.seed = e->seed;
  P.lay = e->lay;
  section_moves_kernel<<<e->grid, e->block, e->lay.total * 8, e->stream>>>(P);
  e->launches++;
  CU(cudaGetLastError());
  if (records) {
    CU(cudaMemcpyAsync(records, d_rec, sizeof(pimc_move_record) * (size_t)e->nrep * nattempt,
                       cudaMemcpyDeviceToHost, e->stream));
    CU(cudaFreeAsync(d_rec, e->stream));
    CU(cudaStreamSynchronize(e->stream));
  }
  return PIMC_OK;
}

int pimc_replica_status(pimc_engine* e, int64_t* accepted, int64_t* attempted, uint32_t* status) {
  if (!e) return fail(PIMC_ERR_INVALID, "null engine");
  std::vector<DevState> st(e->nrep);
  CU(cudaMemcpyAsync(st.data(), e->d_state.p, e->nrep * sizeof(DevState), cudaMemcpyDeviceToHost,
                     e->stream));
  CU(cudaStreamSynchronize(e->stream));
  for (int r = 0; r < e->nrep; ++r) {
    if (accepted) accepted[r] = st[r].accepted;
    if (attempted) attempted[r] = st[r].attempted;
    if (status) status[r] = st[r].status;
  }
  return PIMC_OK;
}

int pimc_node_scale(pimc_engine* e, int replica, int ispec, double* scale) {
  if (!e || replica < 0 || replica >= e->nrep || ispec < 0 || ispec >= kMaxSpecies || !scale)
    return fail(PIMC_ERR_INVALID, "bad argument");
  DevState st;
  CU(cudaMemcpyAsync(&st, e->d_state.p + replica, sizeof(DevState), cudaMemcpyDeviceToHost,
                     e->stream));
  CU(cudaStreamSynchronize(e->stream));
  *scale = st.node_scale[ispec];
  return PIMC_OK;
}

int pimc_thermo_energy(pimc_engine* e, double* host_energy) {
  if (!e || !host_energy) return fail(PIMC_ERR_INVALID, "null argument");
  int maxm = 0;
  for (const DevSys& d : e->hsys) maxm = std::max(maxm, d.nslice);
  const int nchunk = std::max(1, std::min(64, maxm / 8));
  double* d_part = nullptr;
  CU(cudaMallocAsync(&d_part, sizeof(double) * (size_t)e->nrep * nchunk, e->stream));
  ThermoParams P;
  P.sys = e->d_sys.p;
  P.paths = e->d_paths.p;
  P.partial = d_part;
  P.nchunk = nchunk;
  P.nrep = e->nrep;
  P.lay = e->lay;
  thermo_kernel<<<dim3(nchunk, e->nrep), kBlock, e->lay.total * 8, e->stream>>>(P);
  e->launches++;
  CU(cudaGetLastError());
  std::vector<double> part((size_t)e->nrep * nchunk);
  CU(cudaMemcpyAsync(part.data(), d_part, part.size() * 8, cudaMemcpyDeviceToHost, e->stream));
  CU(cudaFreeAsync(d_part, e->stream));
  CU(cudaStreamSynchronize(e->stream));
  for (int r = 0; r < e->nrep; ++r) {
    double s = 0;
    for (int c = 0; c < nchunk; ++c) s += part[(size_t)r * nchunk + c];
    host_energy[r] = s / e->hsys[r].nslice;
  }
  return PIMC_OK;
}

int pimc_action_difference(pimc_engine* e, int level, int nbatch, const double* section,
                           const double* moving, const int* ipart, double* ds) {
  if (!e || nbatch <= 0 || !section || !moving || !ipart || !ds)
    return fail(PIMC_ERR_INVALID, "bad argument");
  const DevSys& s = e->hsys[0];
  if (level < 0 || level > s.nlevel) return fail(PIMC_ERR_INVALID, "level out of range");
  for (int b = 0; b < nbatch; ++b)
    if (ipart[b] < 0 || ipart[b] >= s.npart) return fail(PIMC_ERR_INVALID, "ipart out of range");
  const size_t nsecd = (size_t)nbatch * s.nsec * s.npart * 3, nmovd = (size_t)nbatch * s.nsec * 3;
  double *d_sec = nullptr, *d_mov = nullptr, *d_ds = nullptr;
  int* d_ip = nullptr;
  CU(cudaMallocAsync(&d_sec, nsecd * 8, e->stream));
  CU(cudaMallocAsync(&d_mov, nmovd * 8, e->stream));
  CU(cudaMallocAsync(&d_ds, nbatch * 8, e->stream));
  CU(cudaMallocAsync(&d_ip, nbatch * 4, e->stream));
  CU(cudaMemcpyAsync(d_sec, section, nsecd * 8, cudaMemcpyHostToDevice, e->stream));
  CU(cudaMemcpyAsync(d_mov, moving, nmovd * 8, cudaMemcpyHostToDevice, e->stream));
  CU(cudaMemcpyAsync(d_ip, ipart, nbatch * 4, cudaMemcpyHostToDevice, e->stream));
  ActionDiffParams P;
  P.sys = e->d_sys.p;
  P.section = d_sec;
  P.moving = d_mov;
  P.ipart = d_ip;
  P.ds = d_ds;
  P.level = level;
  P.lay = e->lay;
  action_diff_kernel<<<nbatch, kBlock, e->lay.total * 8, e->stream>>>(P);
  e->launches++;
  CU(cudaGetLastError());
  CU(cudaMemcpyAsync(ds, d_ds, nbatch * 8, cudaMemcpyDeviceToHost, e->stream));
  CU(cudaFreeAsync(d_sec, e->stream));
  CU(cudaFreeAsync(d_mov, e->stream));
  CU(cudaFreeAsync(d_ds, e->stream));
  CU(cudaFreeAsync(d_ip, e->stream));
  CU(cudaStreamSynchronize(e->stream));
  return PIMC_OK;
}

int pimc_node_evaluate(pimc_engine* e, int ispec, int nbatch, const double* r1, const double* r2,
                       double* det, double* d1, double* d2, int* err) {
  if (!e || nbatch <= 0 || !r1 || !r2 || !det || !d1 || !d2 || !err)
    return fail(PIMC_ERR_INVALID, "bad argument");
  const DevSys& s = e->hsys[0];
  if (ispec < 0 || ispec >= s.nspecies || !s.node_kind[ispec])
    return fail(PIMC_ERR_INVALID, "species has no node model");
  const int np = s.npart, n = s.spec_count[ispec];
  const size_t nr = (size_t)nbatch * np * 3;
  double *d_r1, *d_r2, *d_det, *d_d1, *d_d2;
  int* d_err;
  CU(cudaMallocAsync(&d_r1, nr * 8, e->stream));
  CU(cudaMallocAsync(&d_r2, nr * 8, e->stream));
  CU(cudaMallocAsync(&d_det, nbatch * 8, e->stream));
  CU(cudaMallocAsync(&d_d1, (size_t)nbatch * np * 8, e->stream));
  CU(cudaMallocAsync(&d_d2, (size_t)nbatch * np * 8, e->stream));
  CU(cudaMallocAsync(&d_err, nbatch * 4, e->stream));
  CU(cudaMemcpyAsync(d_r1, r1, nr * 8, cudaMemcpyHostToDevice, e->stream));
  CU(cudaMemcpyAsync(d_r2, r2, nr * 8, cudaMemcpyHostToDevice, e->stream));
  NodeEvalParams P;
  P.sys = e->d_sys.p;
  P.state = e->d_state.p;
  P.r1 = d_r1;
  P.r2 = d_r2;
  P.det = d_det;
  P.d1 = d_d1;
  P.d2 = d_d2;
  P.err = d_err;
  P.ispec = ispec;
  P.lay = e->lay;
  const int smem = (8 * np + node_group_scratch(n) + 2) * 8;
  cudaFuncSetAttribute(node_eval_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  node_eval_kernel<<<nbatch, kBlock, smem, e->stream>>>(P);
  e->launches++;
  CU(cudaGetLastError());
  CU(cudaMemcpyAsync(det, d_det, nbatch * 8, cudaMemcpyDeviceToHost, e->stream));
  CU(cudaMemcpyAsync(d1, d_d1, (size_t)nbatch * np * 8, cudaMemcpyDeviceToHost, e->stream));
  CU(cudaMemcpyAsync(d2, d_d2, (size_t)nbatch * np * 8, cudaMemcpyDeviceToHost, e->stream));
  CU(cudaMemcpyAsync(err, d_err, nbatch * 4, cudaMemcpyDeviceToHost, e->stream));
  for (void* p : {(void*)d_r1, (void*)d_r2, (void*)d_det, (void*)d_d1, (void*)d_d2, (void*)d_err})
    CU(cudaFreeAsync(p, e->stream));
  CU(cudaStreamSynchronize(e->stream));
  return PIMC_OK;
}

int pimc_stream_sample(uint64_t seed, uint32_t replica, uint32_t attempt, int n,
                       double* uniforms, double* normals) {
  if (n <= 0 || !uniforms || !normals) return fail(PIMC_ERR_INVALID, "bad argument");
  int nsm = 0;
  if (int rc = device_check(nsm)) return rc;
  double* d = nullptr;
  CU(cudaMalloc(&d, 2 * (size_t)n * sizeof(double)));
  stream_sample_kernel<<<(n + 127) / 128, 128>>>(seed, replica, attempt, n, d, d + n);
  CU(cudaGetLastError());
  CU(cudaMemcpy(uniforms, d, n * sizeof(double), cudaMemcpyDeviceToHost));
  CU(cudaMemcpy(normals, d + n, n * sizeof(double), cudaMemcpyDeviceToHost));
  CU(cudaFree(d));
  return PIMC_OK;
}

int pimc_fp64_peak(double* tflops) {
  if (!tflops) return fail(PIMC_ERR_INVALID, "null argument");
  int nsm = 0;
  if (int rc = device_check(nsm)) return rc;
  double* d = nullptr;
  CU(cudaMalloc(&d, sizeof(double)));
  const int iters = 4096, blocks = nsm * 8, threads = 256;
  fp64_probe_kernel<<<blocks, threads>>>(d, 16);
  cudaEvent_t a, b;
  CU(cudaEventCreate(&a));
  CU(cudaEventCreate(&b));
  float best = 1e30f;
  for (int rep = 0; rep < 5; ++rep) {
    CU(cudaEventRecord(a));
    fp64_probe_kernel<<<blocks, threads>>>(d, iters);
    CU(cudaEventRecord(b));
    CU(cudaEventSynchronize(b));
    float ms = 0;
    CU(cudaEventElapsedTime(&ms, a, b));
    best = std::min(best, ms);
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(d);
  *tflops = 2.0 * 8.0 * iters * (double)blocks * threads / (best * 1e-3) / 1e12;
  return PIMC_OK;
}

int64_t pimc_kernel_launches(pimc_engine* e) { return e ? e->launches : 0; }

// Allocation-free node evaluation.  The device address of the static scratch
// array is looked up once per device (cudaGetSymbolAddress, with that device
// current) on the first call made on it, and cached.
namespace {
constexpr int kMaxDevices = 64;
double* g_noalloc_addr[kMaxDevices] = {nullptr};
}  // namespace

int pimc_node_evaluate_noalloc(const pimc_system* sys, int ispec, double scale, int nbatch,
                               const double* r1, const double* r2, double* det, double* d1,
                               double* d2, int* err, void* stream) {
  if (!sys || nbatch <= 0 || !r1 || !r2 || !det || !d1 || !d2 || !err)
    return fail(PIMC_ERR_INVALID, "bad argument");
  if (int rc = validate(*sys)) return rc;
  if (ispec < 0 || ispec >= sys->nspecies || !sys->node_kind[ispec])
    return fail(PIMC_ERR_INVALID, "species has no node model");
  if (sys->spec_count[ispec] > kMaxNs)
    return fail(PIMC_ERR_CAPACITY, "node species larger than 32 particles (scratch slot limit)");
  int dev = 0;
  CU(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return fail(PIMC_ERR_CAPACITY, "device ordinal beyond 63");
  if (!g_noalloc_addr[dev]) {
    void* p = nullptr;
    CU(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    g_noalloc_addr[dev] = (double*)p;
  }
  NoAllocParams P;
  fill_sys(*sys, P.sys);
  P.r1 = r1;
  P.r2 = r2;
  P.det = det;
  P.d1 = d1;
  P.d2 = d2;
  P.err = err;
  P.scale = scale;
  P.ispec = ispec;
  P.nbatch = nbatch;
  P.scratch = g_noalloc_addr[dev];
  const int grid = nbatch < kNoAllocSlots ? nbatch : kNoAllocSlots;
  const size_t smem = 6 * (size_t)sys->npart * sizeof(double);
  if (smem > 48 * 1024) return fail(PIMC_ERR_CAPACITY, "npart beyond 1024");
  node_eval_noalloc_kernel<<<grid, 32, smem, (cudaStream_t)stream>>>(P);
  CU(cudaGetLastError());
  return PIMC_OK;
}

}  // extern "C"
