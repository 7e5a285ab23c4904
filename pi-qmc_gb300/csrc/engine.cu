// Host side of the engine: the C ABI declared in include/pimc_gb300.h.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/pimc_gb300.h"
#include "entry_kernels.cuh"
#include "kernels.cuh"
#include "noalloc_kernel.cuh"
#include "displace_kernel.cuh"
#include "prefill_kernel.cuh"

namespace pimc {
// register-budget variants of the section kernel (section_variants.cu)
cudaError_t section_launch_v1(int, int, size_t, cudaStream_t, const RunParams&);
cudaError_t section_launch_v2(int, int, size_t, cudaStream_t, const RunParams&);
cudaError_t section_launch_v3(int, int, size_t, cudaStream_t, const RunParams&);
cudaError_t section_launch_v4(int, int, size_t, cudaStream_t, const RunParams&);
int section_occupancy_v1(int, size_t);
int section_occupancy_v2(int, size_t);
int section_occupancy_v3(int, size_t);
int section_occupancy_v4(int, size_t);
void section_smem_cap_v1(int);
void section_smem_cap_v2(int);
void section_smem_cap_v3(int);
void section_smem_cap_v4(int);
// the same without the fixed-node phases (launches without node models)
cudaError_t section_launch_nf_v2(int, int, size_t, cudaStream_t, const RunParams&);
cudaError_t section_launch_nf_v3(int, int, size_t, cudaStream_t, const RunParams&);
cudaError_t section_launch_nf_v4(int, int, size_t, cudaStream_t, const RunParams&);
int section_occupancy_nf_v2(int, size_t);
int section_occupancy_nf_v3(int, size_t);
int section_occupancy_nf_v4(int, size_t);
void section_smem_cap_nf_v2(int);
void section_smem_cap_nf_v3(int);
void section_smem_cap_nf_v4(int);
}  // namespace pimc

using namespace pimc;

namespace {
// minb: 2, 3 or 4 resident 256-thread blocks per SM worth of registers, or 1:
// the 512-thread variant (128 registers)
// nodes: whether a system of the launch has a node model (else the variant
// without the fixed-node phases runs; the 512-thread variant has none)
cudaError_t section_launch(int minb, int grid, int block, size_t smem, cudaStream_t st,
                           const RunParams& P, bool nodes = true) {
  if (minb == 1) return section_launch_v1(grid, block, smem, st, P);
  if (!nodes) {
    if (minb == 3) return section_launch_nf_v3(grid, block, smem, st, P);
    if (minb == 4) return section_launch_nf_v4(grid, block, smem, st, P);
    return section_launch_nf_v2(grid, block, smem, st, P);
  }
  if (minb == 3) return section_launch_v3(grid, block, smem, st, P);
  if (minb == 4) return section_launch_v4(grid, block, smem, st, P);
  return section_launch_v2(grid, block, smem, st, P);
}
int section_occupancy(int minb, int block, size_t smem, bool nodes = true) {
  if (minb == 1) return section_occupancy_v1(block, smem);
  if (!nodes) {
    if (minb == 3) return section_occupancy_nf_v3(block, smem);
    if (minb == 4) return section_occupancy_nf_v4(block, smem);
    return section_occupancy_nf_v2(block, smem);
  }
  if (minb == 3) return section_occupancy_v3(block, smem);
  if (minb == 4) return section_occupancy_v4(block, smem);
  return section_occupancy_v2(block, smem);
}
}  // namespace

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

}  // namespace

namespace pimc {
// Error reporting for the host-only files of the library (paths_io.cc).
int set_error(int code, const std::string& msg) { return fail(code, msg); }
}  // namespace pimc

namespace {

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
      n = 0;
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

// Layout choices the autotuner varies.
struct LayoutOpts {
  bool scratch_global = false;  // per-warp Slater scratch in global memory even when it fits
  bool cold_global = false;     // its cold parts in global memory even when all of it fits
  bool full_ewald_tables = false;  // Ewald tables for every bead (full evalLongRange sums)
};

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
  DevBuf<double> d_prefill_scr;  // global Slater scratch of the cache fill (large matrices)
  DevBuf<long long> d_ekcache;  // structure factors per replica and slice
  DevBuf<long long> d_ekstage;  // per-CTA staging of an attempt's new structure factors
  int ekstage_stride = 0;       // int64 words per CTA
  bool nodes = true;            // a system with a node model (else the kernels without them run)
  DevBuf<double> d_upload;      // pimc_upload_paths: the host paths, before comparison
  DevBuf<unsigned char> d_changed;  // [replica][nslice_max]: slices the upload changed
  DevBuf<double> d_xstage;      // mixed form: per-CTA staging of changed slices' inverses
  long long xstage_cta = 0;     // doubles per CTA
  DevBuf<int> d_order;
  DevBuf<int> d_next;
  DevBuf<double> d_ugrid;
  DevBuf<float> d_ugrid32;
  DevBuf<int> d_kvec;
  DevBuf<double> d_vk;
  // serving: slots over one device pool
  bool server = false;
  pimc_server_config scfg{};
  std::vector<char> active;
  std::vector<long long> slot_path, slot_cache, slot_words;  // pool offsets / sizes (doubles)
  std::map<long long, long long> free_blocks;                // offset -> size (doubles)
  // pair tables on the device, found by content (host address first, then bytes)
  std::multimap<const double*, std::pair<size_t, std::vector<double>>> table_dev;
  size_t table_used = 0;
  DevBuf<double> d_pool;
  DevBuf<int> d_slot_attempts;  // attempts per round of each slot
  std::vector<int> prefill_pending;  // admitted slots whose Slater cache is still empty
  DevBuf<int> d_prefill;
  std::vector<int> slot_attempts;
  bool order_dirty = true;
  int nactive = 0;
  // energy measurement buffers and captured step graphs
  DevBuf<double> d_partial;  // [nrep][kThermoChunks]
  DevBuf<double> d_dscratch;  // displacement moves: node dets and distances per CTA
  DevBuf<double> d_energy;   // [steps][nrep]
  cudaStream_t cap_stream = nullptr;
  cudaGraphExec_t graph = nullptr;
  int graph_attempts = -1, graph_steps = -1;
  Layout lay{};
  Layout est_lay{};  // estimator kernels
  LayoutOpts lay_opts{};
  int ctas_cap = 0;
  int minb = 2;  // register-budget variant of the section kernel
  int block = kBlock;
  int grid = 0;
  int num_sms = 0;
  long long launches = 0;
  ~pimc_engine() {
    if (graph) cudaGraphExecDestroy(graph);
    if (cap_stream) cudaStreamDestroy(cap_stream);
    d_partial.free();
    d_dscratch.free();
    d_energy.free();
    d_sys.free();
    d_state.free();
    d_paths.free();
    d_nodescr.free();
    d_nodecache.free();
    d_ekcache.free();
    d_prefill_scr.free();
    d_ekstage.free();
    d_xstage.free();
    d_upload.free();
    d_changed.free();
    d_order.free();
    d_next.free();
    d_pool.free();
    d_slot_attempts.free();
    d_prefill.free();
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
  if (!(s.tau > 0)) return fail(PIMC_ERR_INVALID, "tau must be positive");
  if (!(s.sigma_factor >= 0) || !(s.dr_sigma_factor >= 0) || !std::isfinite(s.sigma_factor) ||
      !std::isfinite(s.dr_sigma_factor))
    return fail(PIMC_ERR_INVALID, "sigma factors must be finite and non-negative");
  if (s.delayed_rejection && s.mover != PIMC_MOVER_FREE)
    return fail(PIMC_ERR_INVALID, "delayed rejection needs the FreeMover");
  bool fixed = false;
  for (int i = 0; i < s.nspecies; ++i) fixed |= s.node_kind[i] != 0;
  // A section of 2^nlevel + 1 slices may span the whole ring (nslice = 2^nlevel,
  // both ends the same bead, as SectionChooser allows); with fixed nodes the
  // two sections of a double move must each fit.
  if (s.nslice < (1 << s.nlevel) + (fixed ? 1 : 0))
    return fail(PIMC_ERR_INVALID, "nslice smaller than a section");
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
  d.ek_offset = -1;
  d.ek_scale = 1.0;
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
  for (int i = 0; i < s.nspecies; ++i) d.node_dk[i] = std::sqrt(2 * s.spec_mass[i] / s.tau);
  for (int lev = 0; lev < kMaxLevels; ++lev) {
    const int nStride = 1 << lev;
    d.sho_div2[lev] = 1.0 / (2.0 * s.tau * nStride);
    for (int i = 0; i < s.nspecies; ++i) {
      const double lam = 0.5 / s.spec_mass[i];
      d.spr_inv2s2[lev][i] = 0.25 / (lam * s.tau * nStride);
      // FreeMover: sigma = factor sqrt(lambda tau 2^l), factor = defaultSigmaFactor
      // (0 means 1, src/parser/PIMCParser.cc:316-319)
      const double factor = s.sigma_factor != 0 ? s.sigma_factor : 1.0;
      const double sigma = factor * std::sqrt(lam * s.tau * nStride);
      d.mov_sigma[lev][i] = sigma;
      d.mov_inv2s2[lev][i] = 0.5 / (sigma * sigma);
      if (s.delayed_rejection && lev == s.nlevel - 1) {
        // the second proposal: newSigmaFactor (0 means 0.75, PIMCParser.cc:320-322)
        const double nf = s.dr_sigma_factor != 0 ? s.dr_sigma_factor : 0.75;
        const double sg = nf * std::sqrt(lam * s.tau * nStride);
        d.dr_sigma[i] = sg;
        d.dr_inv2s2[i] = 0.5 / (sg * sg);
      }
      if (s.sho_omega[i] > 0) {
        const double wt = s.sho_omega[i] * s.tau * nStride;
        d.sho_cosh[lev][i] = std::cosh(wt);
        d.sho_div1[lev][i] = 1.0 / (2.0 * std::sinh(wt));
        // x coth x - 1 by its series below 0.1 (x^2/3 - x^4/45 + 2x^6/945 - x^8/4725)
        const double x2 = wt * wt;
        const double xc = wt < 0.1 ? x2 * (1.0 / 3 - x2 * (1.0 / 45 - x2 * (2.0 / 945 - x2 / 4725)))
                                   : wt / std::tanh(wt) - 1.0;
        d.sho_a[lev][i] = (float)(s.spec_mass[i] * 0.5 / (s.tau * nStride) * xc);
        d.sho_b[lev][i] = (float)(s.spec_mass[i] * s.sho_omega[i] * std::tanh(0.5 * wt));
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
  d.rcut2_lo = (float)(d.rcut2 * (1.0 - 1e-5));
  d.spring = s.spring;
  d.coulomb = s.coulomb;
  d.ewald = s.ewald;
  d.mover = s.mover;
  d.dr = s.delayed_rejection != 0;
  d.epsilon = s.epsilon > 0 ? s.epsilon : 1.0;
}

// Doubles of one Slater-result cache entry: epoch, determinant, two distance
// vectors, the element matrix (SHO exp values; free-particle nodes add three
// gradient matrices) and a stale-row word, rounded to an even count.
int cache_entry_doubles(const DevSys& d) {
  bool free_nodes = false;
  for (int i = 0; i < d.nspecies; ++i) free_nodes |= d.node_kind[i] == PIMC_NODES_FREE;
  const int n = d.ns_max;
  // + the stale-row word; the mixed form adds, for free-particle nodes, the
  // inverse block (epoch, update count, n*n inverse) that its Sherman-Morrison
  // updates work on (sm_species)
  const bool xblock = d.mixed && free_nodes;
  return (2 + 2 * n + n * n * (free_nodes ? 4 : 1) + 1 + (xblock ? 2 + n * n : 0) + 1) & ~1;
}

// Doubles of inverse-block staging one CTA needs for a replica (mixed form with
// a cache and free-particle nodes).
long long xstage_doubles(const DevSys& d) {
  bool free_nodes = false;
  for (int i = 0; i < d.nspecies; ++i) free_nodes |= d.node_kind[i] == PIMC_NODES_FREE;
  return d.mixed && free_nodes && d.nc_offset >= 0
             ? (long long)d.nsec * (d.ns_max * d.ns_max + 2)
             : 0;
}

// Grows the inverse-block staging to grid CTAs of e->xstage_cta doubles.
int ensure_xstage(pimc_engine* e, int grid) {
  const size_t need = (size_t)grid * e->xstage_cta;
  if (need == 0 || need <= e->d_xstage.n) return PIMC_OK;
  CU(cudaStreamSynchronize(e->stream));
  if (e->d_xstage.alloc(need)) return fail(PIMC_ERR_CUDA, "cudaMalloc inverse staging");
  return PIMC_OK;
}

// Fixed-point exponent of a replica's structure-factor cache, or -1 when it
// has none (no Ewald sum; fixed-node sections that can overlap; charges too
// large for a fine grid): |rho_k| <= sum |q|, and an update adds at most
// 2 max|q| more, so 60 bits cover 3 sum |q|.
int ek_bits(const DevSys& d) {
  if (!(d.ewald && d.coulomb && d.totk > 0)) return -1;
  if (d.fixed_node && !((1 << d.nlevel) < d.nslice / 2)) return -1;
  double qsum = 0;
  for (int i = 0; i < d.nspecies; ++i) qsum += std::fabs(d.charge[i]) * d.spec_count[i];
  const int ebits = 60 - (int)std::ceil(std::log2(std::max(qsum, 1.0)) + 1e-9);
  return ebits < 24 ? -1 : ebits;
}

// Dynamic shared memory of the section-sized kernels (bytes; the opt-in
// maximum is 227 KB, less the kernels' few KB of static shared memory).
constexpr int kSmemLimit = 220 * 1024;

Layout make_layout(const std::vector<DevSys>& sys, int nwarps, bool& ok, LayoutOpts opts = {}) {
  int nsec = 0, np = 0, nsm = 1, per = 0;
  bool fixed = false, ewald_full = false;
  for (const DevSys& d : sys) {
    nsec = std::max(nsec, d.nsec);
    np = std::max(np, d.npart);
    nsm = std::max(nsm, d.ns_max);
    fixed |= d.fixed_node != 0;
    if (d.ewald) {
      per = std::max(per, d.ikmax[0] + 1 + 2 * d.ikmax[1] + 1 + 2 * d.ikmax[2] + 1);
      ewald_full |= opts.full_ewald_tables || ek_bits(d) < 0;
    }
  }
  Layout L{};
  int off = 0;
  auto take = [&](int n) {
    const int o = off;
    off += (n + 1) & ~1;  // keep 16-byte alignment
    return o;
  };
  // Ewald tables: every bead of a slice for a full evalLongRange, or 16 bead
  // columns (8 slices' old and new moving bead) when every Ewald replica keeps
  // its structure factors
  L.ewt_cols = per ? (ewald_full ? np + 1 : std::min(np + 1, 16)) : 0;
  L.s1 = take(3 * nsec * np);
  L.s2 = take(fixed ? 3 * nsec * np : 0);
  L.mv = take(3 * nsec);
  L.nrm = take(3 * nsec);
  L.red = take(64);
  L.vred = take(9 * kWarps);
  L.q = take(np);
  L.dm = take(kMaxSpecies * nsec);
  L.ndm = take(nsec);
  L.dist = take(fixed ? nsec * 2 * nsm : 0);
  L.ndist = take(fixed ? nsec * 2 * nsm : 0);
  L.ewt = take(2 * per * L.ewt_cols);
  L.ictl = take((C_NCTL + 2 * kMaxSpecies * nsec + 1) / 2 + 1);
  bool sho = false;
  for (const DevSys& d : sys)
    for (int i = 0; i < d.nspecies; ++i) sho |= d.node_kind[i] == PIMC_NODES_SHO;
  // exp-matrix cache of the moving species' section slices; left out (the
  // levels then recompute whole matrices) when it would not fit
  // (only systems without the path-resident cache use it)
  bool uncached = false;
  for (const DevSys& d : sys) uncached |= d.fixed_node && !((1 << d.nlevel) < d.nslice / 2);
  L.ecache = (sho && uncached && (off + nsec * nsm * nsm) * 8 <= 120 * 1024)
                 ? take(nsec * nsm * nsm) : -1;
  bool anyfree_col = false;
  for (const DevSys& d : sys)
    for (int i = 0; i < d.nspecies; ++i) anyfree_col |= d.node_kind[i] == PIMC_NODES_FREE;
  L.ncol_stride = nsm * (anyfree_col ? 4 : 1);
  const int ncol_size = fixed ? nsec * L.ncol_stride : 0;
  // per-warp Slater scratch: (32 / W) lane groups of node_group_scratch(n)
  // doubles, or of its hot and cold parts apart (the species present decide
  // it: a smaller species packs more lane groups per warp)
  int full = 0, hot = 0, cold = 0;
  for (const DevSys& d : sys)
    for (int i = 0; i < d.nspecies; ++i)
      if (d.node_kind[i]) {
        const int n = d.spec_count[i], G = 32 / node_group_width(n);
        const bool fr = d.node_kind[i] == PIMC_NODES_FREE;
        full = std::max(full, G * node_group_scratch(n, fr));
        hot = std::max(hot, G * node_group_hot(n));
        cold = std::max(cold, G * node_group_cold(n, fr));
      }
  full = (full + 1) & ~1;
  hot = (hot + 1) & ~1;
  cold = (cold + 1) & ~1;
  const int limit = kSmemLimit / 8;
  const int base = off;
  // placements, best first: everything in shared memory; the LU and inverse
  // in shared memory with the cold parts (and then the new-column buffer) in
  // the CTA's global area; all of the scratch in global memory
  enum { kAll, kHotCol, kHot, kGlobalCol, kGlobal };
  int place = kGlobal;
  if (!fixed) {
    place = kAll;
  } else {
    const int cand[5][3] = {  // {ncol in smem, per-warp scratch in smem, split}
        {1, full, 0}, {1, hot, 1}, {0, hot, 1}, {1, 0, 0}, {0, 0, 0}};
    const int first = opts.scratch_global ? kGlobalCol : (opts.cold_global ? kHotCol : kAll);
    for (int c = first; c <= kGlobal; ++c)
      if (base + (cand[c][0] ? ncol_size : 0) + nwarps * cand[c][1] <= limit || c == kGlobal) {
        place = c;
        break;
      }
  }
  const bool ncol_smem = place == kAll || place == kHotCol || place == kGlobalCol;
  L.ncol = (fixed && ncol_smem) ? take(ncol_size) : -1;
  L.ncol_global = fixed && !ncol_smem;
  L.split = place == kHotCol || place == kHot;
  L.nodescr_in_smem = place == kAll || L.split;
  L.nodescr_stride = place == kAll ? full : (L.split ? hot : full);
  L.nodecold_stride = L.split ? cold : 0;
  L.nodescr = L.nodescr_in_smem ? take(nwarps * L.nodescr_stride) : -1;
  const int gwarp = L.split ? cold : (L.nodescr_in_smem ? 0 : full);
  L.gcta = nwarps * gwarp + (L.ncol_global ? ncol_size : 0);
  L.total = off;
  ok = L.total <= limit;
  return L;
}

void set_smem_caps() {
  section_smem_cap_v1(kSmemLimit);
  section_smem_cap_v2(kSmemLimit);
  section_smem_cap_v3(kSmemLimit);
  section_smem_cap_v4(kSmemLimit);
  section_smem_cap_nf_v2(kSmemLimit);
  section_smem_cap_nf_v3(kSmemLimit);
  section_smem_cap_nf_v4(kSmemLimit);
  cudaFuncSetAttribute(thermo_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemLimit);
  cudaFuncSetAttribute(action_diff_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       kSmemLimit);
}

// Shared memory of the estimator kernels: one staged slice (in the section
// arrays' places), the reduction buffer, charges and the e^{ik.r} tables of the
// largest k-list among the systems' and an estimator's own (ikmax_extra).
Layout estimator_layout(const std::vector<DevSys>& sys, const int* ikmax_extra) {
  int nsec = 1, np = 1, ik[3] = {0, 0, 0};
  for (const DevSys& d : sys) {
    nsec = std::max(nsec, d.nsec);
    np = std::max(np, d.npart);
    if (d.ewald)
      for (int a = 0; a < 3; ++a) ik[a] = std::max(ik[a], d.ikmax[a]);
  }
  if (ikmax_extra)
    for (int a = 0; a < 3; ++a) ik[a] = std::max(ik[a], ikmax_extra[a]);
  Layout L{};
  int off = 0;
  auto take = [&](int n) {
    const int o = off;
    off += (n + 1) & ~1;
    return o;
  };
  L.s1 = take(3 * nsec * np);
  L.s2 = L.s1;
  L.mv = take(3 * nsec);
  L.nrm = L.mv;
  L.red = take(64);
  L.vred = L.red;
  L.q = take(np);
  L.ewt = take(2 * ((ik[0] + 1) + (2 * ik[1] + 1) + (2 * ik[2] + 1)) * (np + 1));
  L.ictl = take(C_NCTL + 2);
  L.dm = L.ndm = L.dist = L.ndist = L.red;
  L.ecache = L.ncol = -1;
  L.nodescr = 0;
  L.nodescr_in_smem = 1;
  L.ewt_cols = np + 1;
  L.split = L.ncol_global = L.gcta = L.nodecold_stride = 0;
  L.total = off;
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

int prefill_ewald(pimc_engine* e, const int* d_slots, int nslot,
                  const unsigned char* changed = nullptr);

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
    d.stream_id = (uint32_t)r;
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
  e->nodes = false;
  for (const DevSys& d : e->hsys) e->nodes |= d.fixed_node != 0;
  bool ok = false;
  e->lay = make_layout(e->hsys, e->block / 32, ok);
  if (!ok) {
    delete e;
    return fail(PIMC_ERR_CAPACITY, "working set does not fit in shared memory");
  }
  e->est_lay = estimator_layout(e->hsys, nullptr);
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
  // launch geometry: persistent grid over replicas.  The dynamic shared-memory
  // cap is the layout limit for every engine (the attribute is per function,
  // shared by all engines of the process).
  set_smem_caps();
  int occ = 1;
  occ = section_occupancy(e->minb, e->block, e->lay.total * 8, e->nodes);
  occ = std::max(occ, 1);
  e->grid = std::min(nrep, nsm * occ);
  for (DevSys& d : e->hsys) d.inv_offset = e->lay.gcta > 0 ? 0 : -1;
  if (e->lay.gcta > 0 && e->d_nodescr.alloc((size_t)e->grid * e->lay.gcta)) {
    delete e;
    return fail(PIMC_ERR_CUDA, "cudaMalloc node scratch");
  }
  // Slater-result cache: per replica, per species, per path slice.  Left out
  // when the two sections of an attempt can overlap (2^L >= M/2).
  {
    long long coff = 0;
    for (DevSys& d : e->hsys) {
      const bool use = d.fixed_node && (1 << d.nlevel) < d.nslice / 2;
      d.nc_stride = cache_entry_doubles(d);
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
    for (const DevSys& d : e->hsys) e->xstage_cta = std::max(e->xstage_cta, xstage_doubles(d));
    if (e->xstage_cta > 0 && e->d_xstage.alloc((size_t)e->grid * e->xstage_cta)) {
      delete e;
      return fail(PIMC_ERR_CUDA, "cudaMalloc inverse staging");
    }
  }
  // Structure-factor cache of Ewald systems (left out, like the Slater cache,
  // when an attempt's two sections can overlap, and when the charges are too
  // large for a fine fixed-point grid).
  {
    long long eoff = 0;
    for (DevSys& d : e->hsys) {
      d.ek_offset = -1;
      if (!(d.ewald && d.coulomb && d.totk > 0)) continue;
      if (d.fixed_node && !((1 << d.nlevel) < d.nslice / 2)) continue;
      double qsum = 0;
      for (int i = 0; i < d.nspecies; ++i) qsum += std::fabs(d.charge[i]) * d.spec_count[i];
      // |rho_k| <= sum |q|; an update adds at most 2 max|q| more: 60 bits cover 3 sum |q|
      const int ebits = 60 - (int)std::ceil(std::log2(std::max(qsum, 1.0)) + 1e-9);
      if (ebits < 24) continue;
      d.ek_scale = std::ldexp(1.0, ebits);
      d.ek_offset = eoff;
      eoff += 2LL * d.nslice * d.totk;
      e->ekstage_stride = std::max(e->ekstage_stride, 2 * (d.nsec - 2) * d.totk);
    }
    if (eoff > 0 && (e->d_ekcache.alloc(eoff) ||
                     e->d_ekstage.alloc((size_t)e->grid * e->ekstage_stride))) {
      delete e;
      return fail(PIMC_ERR_CUDA, "cudaMalloc structure-factor cache");
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
  if (int rc = prefill_ewald(e, nullptr, nrep)) {  // structure factors of the zero paths
    delete e;
    return rc;
  }
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

}  // extern "C"

namespace {
// Fills the Slater-result cache entries of `nslot` replicas (slots on the device,
// or null for 0 .. nslot-1) from their current paths, one warp per entry.
int prefill_cache(pimc_engine* e, double* cache, const int* d_slots, int nslot,
                  bool only_invalid = false) {
  int nsp = 0, mmax = 0, nmax = 0;
  bool anyfree = false, any = false;
  for (int r = 0; r < e->nrep; ++r) {
    const DevSys& d = e->hsys[r];
    if (!(d.fixed_node && d.nc_offset >= 0)) continue;
    any = true;
    nsp = std::max(nsp, d.nspecies);
    mmax = std::max(mmax, d.nslice);
    for (int i = 0; i < d.nspecies; ++i)
      if (d.node_kind[i]) {
        nmax = std::max(nmax, d.spec_count[i]);
        anyfree |= d.node_kind[i] == PIMC_NODES_FREE;
      }
  }
  if (!any || nslot == 0) return PIMC_OK;
  PrefillParams P;
  P.sys = e->d_sys.p;
  P.state = e->d_state.p;
  P.paths = e->server ? e->d_pool.p : e->d_paths.p;
  P.cache = cache;
  P.slots = d_slots;
  P.nslot = nslot;
  P.only_invalid = only_invalid ? 1 : 0;
  P.ntask_per_slot = nsp * mmax;
  P.stage_stride = (6 * nmax + 1) & ~1;
  // Slater scratch: all of it in shared memory up to 6 KB a warp; else its hot
  // part (LU, inverse) there up to 24 KB with the cold part in global memory;
  // else all of it in global memory
  const int full = (node_group_scratch(nmax, anyfree) + 1) & ~1;
  const int hot = (node_group_hot(nmax) + 1) & ~1;
  const int cold = (node_group_cold(nmax, anyfree) + 1) & ~1;
  const bool all_smem = full * 8 <= 6 * 1024, split = !all_smem && hot * 8 <= 24 * 1024;
  P.scratch_stride = split ? hot : full;
  P.cold_stride = split ? cold : 0;
  const int nw = kBlock / 32;
  const size_t smem =
      (size_t)nw * (P.stage_stride + ((all_smem || split) ? P.scratch_stride : 0)) * 8;
  const long long ntask = (long long)nslot * P.ntask_per_slot;
  const int grid = (int)std::min<long long>((ntask + nw - 1) / nw, (long long)e->num_sms * 4);
  P.gscratch = nullptr;
  P.gcold = nullptr;
  const size_t gper = all_smem ? 0 : (split ? (size_t)cold : (size_t)full);
  if (gper) {
    const size_t need = (size_t)grid * nw * gper;
    if (e->d_prefill_scr.n < need) {
      CU(cudaStreamSynchronize(e->stream));  // an earlier fill may still use it
      if (e->d_prefill_scr.alloc(need)) return fail(PIMC_ERR_CUDA, "cudaMalloc prefill scratch");
    }
    if (split)
      P.gcold = e->d_prefill_scr.p;
    else
      P.gscratch = e->d_prefill_scr.p;
  }
  cudaFuncSetAttribute(cache_prefill_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       200 * 1024);
  cache_prefill_kernel<<<grid, kBlock, smem, e->stream>>>(P);
  e->launches++;
  CU(cudaGetLastError());
  return PIMC_OK;
}

// Fills the structure-factor cache of `nslot` replicas (device slot list, or
// null for 0 .. nslot-1) from their current paths.
int prefill_ewald(pimc_engine* e, const int* d_slots, int nslot, const unsigned char* changed) {
  if (!e->d_ekcache.p || nslot == 0) return PIMC_OK;
  int mmax = 0, np = 0, per = 0;
  for (const DevSys& d : e->hsys) {
    if (d.ek_offset < 0) continue;
    mmax = std::max(mmax, d.nslice);
    np = std::max(np, d.npart);
    per = std::max(per, d.ikmax[0] + 1 + 2 * d.ikmax[1] + 1 + 2 * d.ikmax[2] + 1);
  }
  if (mmax == 0) return PIMC_OK;
  EkPrefillParams P;
  P.sys = e->d_sys.p;
  P.paths = e->d_paths.p;
  P.ek = e->d_ekcache.p;
  P.slots = d_slots;
  P.nslot = nslot;
  P.nslice_max = mmax;
  P.changed = changed;
  const size_t smem = (size_t)per * np * 16 + (size_t)np * 8;
  if (smem > 200 * 1024) return fail(PIMC_ERR_CAPACITY, "Ewald tables exceed shared memory");
  cudaFuncSetAttribute(ewald_prefill_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       200 * 1024);
  ewald_prefill_kernel<<<dim3(mmax, nslot), kBlock, smem, e->stream>>>(P);
  e->launches++;
  CU(cudaGetLastError());
  return PIMC_OK;
}
}  // namespace

extern "C" {

// The upload lands in a staging buffer; a kernel compares it with the
// engine's paths slice by slice, copies the slices that differ and flags
// them, and only the cached results that depend on a changed slice (Slater
// entries pairing it, its structure factors) are rebuilt.  The caches are
// consistent with the engine's paths after every call (moves keep them so),
// so the rebuilt and kept entries together equal a full rebuild bit for bit.
int pimc_upload_paths(pimc_engine* e, const double* host_xyz) {
  if (!e || !host_xyz) return fail(PIMC_ERR_INVALID, "null argument");
  if (e->server) return fail(PIMC_ERR_INVALID, "a server takes paths at admission");
  const size_t n = e->path_off[e->nrep];
  int mmax = 1;
  for (const DevSys& d : e->hsys) mmax = std::max(mmax, d.nslice);
  const size_t nflag = (size_t)e->nrep * mmax;
  if (e->d_upload.n < n || e->d_changed.n < nflag) {
    CU(cudaStreamSynchronize(e->stream));
    if ((e->d_upload.n < n && e->d_upload.alloc(n)) ||
        (e->d_changed.n < nflag && e->d_changed.alloc(nflag))) {
      // no room for the staging copy: copy in place and rebuild every cache
      cudaGetLastError();  // (the failed allocation's error is handled here)
      e->d_upload.free();
      e->d_changed.free();
      CU(cudaMemcpyAsync(e->d_paths.p, host_xyz, n * sizeof(double), cudaMemcpyHostToDevice,
                         e->stream));
      const dim3 grid(16, (unsigned)std::min(e->nrep, 65535));
      path_scan_kernel<<<grid, kBlock, 0, e->stream>>>(e->d_sys.p, e->d_state.p, e->d_paths.p,
                                                       e->nrep);
      CU(cudaGetLastError());
      e->launches++;
      if (e->d_nodecache.p) {
        CU(cudaMemsetAsync(e->d_nodecache.p, 0xff, e->d_nodecache.n * sizeof(double),
                           e->stream));
        if (int rc = prefill_cache(e, e->d_nodecache.p, nullptr, e->nrep)) return rc;
      }
      return prefill_ewald(e, nullptr, e->nrep);
    }
  }
  CU(cudaMemcpyAsync(e->d_upload.p, host_xyz, n * sizeof(double), cudaMemcpyHostToDevice,
                     e->stream));
  {
    const dim3 grid((unsigned)mmax, (unsigned)std::min(e->nrep, 65535));
    path_update_kernel<<<grid, 128, 0, e->stream>>>(e->d_sys.p, e->d_paths.p, e->d_upload.p,
                                                    e->d_changed.p, mmax, e->nrep);
    CU(cudaGetLastError());
    e->launches++;
  }
  {
    const dim3 grid(16, (unsigned)std::min(e->nrep, 65535));
    path_scan_kernel<<<grid, kBlock, 0, e->stream>>>(e->d_sys.p, e->d_state.p, e->d_paths.p,
                                                     e->nrep);
    CU(cudaGetLastError());
    e->launches++;
  }
  if (e->d_nodecache.p) {
    const dim3 grid(8, (unsigned)std::min(e->nrep, 65535));
    cache_invalidate_kernel<<<grid, 128, 0, e->stream>>>(e->d_sys.p, e->d_nodecache.p,
                                                         e->d_changed.p, mmax, e->nrep);
    CU(cudaGetLastError());
    e->launches++;
    if (int rc = prefill_cache(e, e->d_nodecache.p, nullptr, e->nrep, true)) return rc;
  }
  return prefill_ewald(e, nullptr, e->nrep, e->d_changed.p);
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

}  // extern "C"

namespace {
// Device address and shape of replica r's path (an active slot on a server).
int replica_path(pimc_engine* e, int r, double** dev, int* npart, int* nslice) {
  if (!e || r < 0 || r >= e->nrep) return fail(PIMC_ERR_INVALID, "bad replica");
  if (e->server && !e->active[r]) return fail(PIMC_ERR_INVALID, "slot not in use");
  const DevSys& d = e->hsys[r];
  *dev = (e->server ? e->d_pool.p : e->d_paths.p) + d.path_offset;
  *npart = d.npart;
  *nslice = d.nslice;
  return PIMC_OK;
}

// Rebuilds replica r's Slater-result cache from its current path and state.
int refresh_cache(pimc_engine* e, int r) {
  const DevSys& d = e->hsys[r];
  const bool slater = d.fixed_node && d.nc_offset >= 0, ewald = !e->server && d.ek_offset >= 0;
  if (!slater && !ewald) return PIMC_OK;
  if (e->d_prefill.n < 1 && e->d_prefill.alloc(64))
    return fail(PIMC_ERR_CUDA, "cudaMalloc prefill list");
  CU(cudaMemcpyAsync(e->d_prefill.p, &r, sizeof(int), cudaMemcpyHostToDevice, e->stream));
  if (slater) {
    double* base = e->server ? e->d_pool.p : e->d_nodecache.p;
    CU(cudaMemsetAsync(base + d.nc_offset, 0xff,
                       (size_t)d.nspecies * d.nslice * d.nc_stride * sizeof(double), e->stream));
    if (int rc = prefill_cache(e, base, e->d_prefill.p, 1)) return rc;
  }
  return ewald ? prefill_ewald(e, e->d_prefill.p, 1) : PIMC_OK;
}
}  // namespace

extern "C" {

int pimc_write_paths(pimc_engine* e, int replica, const char* filename) {
  double* dev;
  int npart, nslice;
  if (int rc = replica_path(e, replica, &dev, &npart, &nslice)) return rc;
  std::vector<double> h((size_t)npart * nslice * 3);
  CU(cudaMemcpyAsync(h.data(), dev, h.size() * sizeof(double), cudaMemcpyDeviceToHost,
                     e->stream));
  CU(cudaStreamSynchronize(e->stream));
  return pimc_paths_write_file(filename, h.data(), npart, nslice);
}

int pimc_read_paths(pimc_engine* e, int replica, const char* filename, int bfactor) {
  double* dev;
  int npart, nslice;
  if (int rc = replica_path(e, replica, &dev, &npart, &nslice)) return rc;
  if (e->server) return fail(PIMC_ERR_INVALID, "a server takes paths at admission");
  std::vector<double> h((size_t)npart * nslice * 3);
  if (int rc = pimc_paths_read_file(filename, h.data(), npart, nslice, bfactor)) return rc;
  CU(cudaMemcpyAsync(dev, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice,
                     e->stream));
  if (int rc = refresh_cache(e, replica)) return rc;
  CU(cudaStreamSynchronize(e->stream));  // h goes out of scope
  return PIMC_OK;
}

int pimc_get_replica_state(pimc_engine* e, int replica, pimc_replica_state* out) {
  double* dev;
  int npart, nslice;
  if (int rc = replica_path(e, replica, &dev, &npart, &nslice)) return rc;
  if (!out) return fail(PIMC_ERR_INVALID, "null argument");
  DevState st;
  CU(cudaMemcpyAsync(&st, e->d_state.p + replica, sizeof(DevState), cudaMemcpyDeviceToHost,
                     e->stream));
  CU(cudaStreamSynchronize(e->stream));
  memset(out, 0, sizeof(*out));
  out->attempt = st.attempt;
  out->status = st.status;
  out->accepted = st.accepted;
  out->attempted = st.attempted;
  for (int k = 0; k < PIMC_MAX_SPECIES; ++k) out->node_scale[k] = st.node_scale[k];
  return PIMC_OK;
}

int pimc_set_replica_state(pimc_engine* e, int replica, const pimc_replica_state* in) {
  double* dev;
  int npart, nslice;
  if (int rc = replica_path(e, replica, &dev, &npart, &nslice)) return rc;
  if (!in) return fail(PIMC_ERR_INVALID, "null argument");
  for (int k = 0; k < PIMC_MAX_SPECIES; ++k)
    if (!(in->node_scale[k] > 0) || !std::isfinite(in->node_scale[k]))
      return fail(PIMC_ERR_INVALID, "node scales must be positive and finite");
  DevState st;
  CU(cudaMemcpyAsync(&st, e->d_state.p + replica, sizeof(DevState), cudaMemcpyDeviceToHost,
                     e->stream));
  CU(cudaStreamSynchronize(e->stream));
  st.attempt = in->attempt;
  st.status = in->status;
  st.accepted = in->accepted;
  st.attempted = in->attempted;
  for (int k = 0; k < kMaxSpecies; ++k) {
    if (st.node_scale[k] != in->node_scale[k]) st.epoch[k]++;
    st.node_scale[k] = in->node_scale[k];
  }
  CU(cudaMemcpyAsync(e->d_state.p + replica, &st, sizeof(DevState), cudaMemcpyHostToDevice,
                     e->stream));
  // cached Slater results were made at the old scales
  if (int rc = refresh_cache(e, replica)) return rc;
  CU(cudaStreamSynchronize(e->stream));
  return PIMC_OK;
}

namespace {
constexpr int kThermoChunks = 64;

// Enqueues the energy measurement of every replica into d_energy[row][*].
int enqueue_thermo(pimc_engine* e, cudaStream_t st, int row) {
  if (e->d_partial.n < (size_t)e->nrep * kThermoChunks &&
      e->d_partial.alloc((size_t)e->nrep * kThermoChunks))
    return fail(PIMC_ERR_CUDA, "cudaMalloc energy partials");
  if (e->d_energy.n < (size_t)(row + 1) * e->nrep) {
    DevBuf<double> bigger;
    if (bigger.alloc((size_t)(row + 1) * e->nrep)) return fail(PIMC_ERR_CUDA, "cudaMalloc energies");
    std::swap(bigger.p, e->d_energy.p);
    std::swap(bigger.n, e->d_energy.n);
  }
  ThermoParams P;
  P.sys = e->d_sys.p;
  P.index = nullptr;
  P.paths = e->d_paths.p;
  P.ekcache = e->d_ekcache.p;
  P.partial = e->d_partial.p;
  P.nchunk = kThermoChunks;
  P.nrep = e->nrep;
  P.lay = e->est_lay;
  thermo_kernel<<<dim3(kThermoChunks, e->nrep), kBlock, e->est_lay.total * 8, st>>>(P);
  thermo_reduce_kernel<<<(e->nrep + 127) / 128, 128, 0, st>>>(
      e->d_sys.p, nullptr, e->d_partial.p, kThermoChunks, e->nrep,
      e->d_energy.p + (size_t)row * e->nrep);
  e->launches += 2;
  CU(cudaGetLastError());
  return PIMC_OK;
}

void fill_run_params(pimc_engine* e, RunParams& P, int nattempt, pimc_move_record* d_rec) {
  P.sys = e->d_sys.p;
  P.state = e->d_state.p;
  P.paths = e->d_paths.p;
  P.nodescr_g = e->d_nodescr.p;
  P.nodecache = e->d_nodecache.p;
  P.ekcache = e->d_ekcache.p;
  P.ekstage = e->d_ekstage.p;
  P.ekstage_stride = e->ekstage_stride;
  P.xstage = e->xstage_cta > 0 ? e->d_xstage.p : nullptr;
  P.xstage_cta = e->xstage_cta;
  P.rec = d_rec;
  P.order = e->d_order.p;
  P.next = e->d_next.p;
  P.nattempt = nattempt;
  P.nattempt_r = nullptr;
  P.nrep = e->nrep;
  P.seed = e->seed;
  P.lay = e->lay;
}
}  // namespace

int pimc_run_sections(pimc_engine* e, int nattempt, pimc_move_record* records) {
  if (!e || nattempt < 0) return fail(PIMC_ERR_INVALID, "bad argument");
  if (nattempt == 0) return PIMC_OK;
  pimc_move_record* d_rec = nullptr;
  if (records) {
    CU(cudaMallocAsync(&d_rec, sizeof(pimc_move_record) * (size_t)e->nrep * nattempt, e->stream));
    CU(cudaMemsetAsync(d_rec, 0, sizeof(pimc_move_record) * (size_t)e->nrep * nattempt, e->stream));
  }
  RunParams P;
  fill_run_params(e, P, nattempt, d_rec);
  CU(cudaMemsetAsync(e->d_next.p, 0, sizeof(int), e->stream));
  CU(section_launch(e->minb, e->grid, e->block, e->lay.total * 8, e->stream, P, e->nodes));
  e->launches++;
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
  if (e->server) return fail(PIMC_ERR_INVALID, "use pimc_server_energy on a server");
  if (int rc = enqueue_thermo(e, e->stream, 0)) return rc;
  CU(cudaMemcpyAsync(host_energy, e->d_energy.p, e->nrep * sizeof(double),
                     cudaMemcpyDeviceToHost, e->stream));
  CU(cudaStreamSynchronize(e->stream));
  return PIMC_OK;
}

namespace {
// Runs one estimator kernel over every replica (64 chunks each), reduces the
// partials per replica (÷ M) and copies the energies to the host.
enum { kEstVirial = 0, kEstCoulomb = 1 };
int run_estimator(pimc_engine* e, int which, EstimatorParams P, const Layout& L, double* host) {
  if (e->d_partial.n < (size_t)e->nrep * kThermoChunks &&
      e->d_partial.alloc((size_t)e->nrep * kThermoChunks))
    return fail(PIMC_ERR_CUDA, "cudaMalloc energy partials");
  double* d_out = nullptr;
  CU(cudaMallocAsync(&d_out, e->nrep * sizeof(double), e->stream));
  P.sys = e->d_sys.p;
  P.paths = e->d_paths.p;
  P.partial = e->d_partial.p;
  P.nchunk = kThermoChunks;
  P.nrep = e->nrep;
  P.lay = L;
  const dim3 grid(kThermoChunks, e->nrep);
  if (which == kEstVirial) {
    cudaFuncSetAttribute(virial_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    virial_kernel<<<grid, kBlock, L.total * 8, e->stream>>>(P);
  } else {
    cudaFuncSetAttribute(coulomb_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    coulomb_kernel<<<grid, kBlock, L.total * 8, e->stream>>>(P);
  }
  thermo_reduce_kernel<<<(e->nrep + 127) / 128, 128, 0, e->stream>>>(
      e->d_sys.p, nullptr, e->d_partial.p, kThermoChunks, e->nrep, d_out);
  e->launches += 2;
  CU(cudaGetLastError());
  CU(cudaMemcpyAsync(host, d_out, e->nrep * sizeof(double), cudaMemcpyDeviceToHost, e->stream));
  CU(cudaFreeAsync(d_out, e->stream));
  CU(cudaStreamSynchronize(e->stream));
  return PIMC_OK;
}
}  // namespace

int pimc_run_displace(pimc_engine* e, int nattempt, const double* box, int nmoving, int species,
                      pimc_displace_record* records) {
  if (!e || e->server || nattempt < 0 || !box || nmoving < 1 || nmoving > kMaxMoving)
    return fail(PIMC_ERR_INVALID, "bad argument");
  for (const DevSys& d : e->hsys) {
    if (species >= d.nspecies) return fail(PIMC_ERR_INVALID, "species out of range");
    const int pool = species < 0 ? d.npart : d.spec_count[species];
    if (nmoving > pool) return fail(PIMC_ERR_INVALID, "more moving particles than candidates");
    if (d.fixed_node && (d.nslice % 2)) return fail(PIMC_ERR_INVALID, "odd nslice");
  }
  if (nattempt == 0) return PIMC_OK;
  // shared memory: a section layout (slices staged for the Ewald sums, the
  // reduction buffer, charges, control words, Slater scratch) plus a slice-pair
  // staging area per lane group
  const int dthreads = std::min(e->block, kBlock), nwarps = dthreads / 32;
  int stage = 0, half_max = 1, nsm = 1;
  for (const DevSys& d : e->hsys) {
    half_max = std::max(half_max, d.nslice / 2);
    nsm = std::max(nsm, d.ns_max);
    for (int i = 0; i < d.nspecies; ++i)
      if (d.node_kind[i]) {
        const int n = d.spec_count[i];
        stage = std::max(stage, (32 / node_group_width(n)) * 6 * n);
      }
  }
  // (full Ewald tables: every slice's evalLongRange is summed here)
  LayoutOpts dopt;
  dopt.full_ewald_tables = true;
  bool lok = false;
  Layout L = make_layout(e->hsys, nwarps, lok, dopt);
  if (!lok || (size_t)(L.total + nwarps * stage) * 8 > (size_t)kSmemLimit) {
    dopt.scratch_global = true;
    L = make_layout(e->hsys, nwarps, lok, dopt);
  }
  const int stage_off = L.total;
  const size_t smem = (size_t)(L.total + nwarps * stage) * 8;
  if (!lok || smem > (size_t)kSmemLimit)
    return fail(PIMC_ERR_CAPACITY, "displacement working set too large");
  if ((size_t)e->grid * L.gcta > e->d_nodescr.n) {
    CU(cudaStreamSynchronize(e->stream));
    if (e->d_nodescr.alloc((size_t)e->grid * L.gcta))
      return fail(PIMC_ERR_CUDA, "cudaMalloc node scratch");
  }
  const long long sstride = (long long)half_max * (1 + 4 * nsm);
  const size_t need = (size_t)e->grid * sstride;
  if (e->d_dscratch.n < need && e->d_dscratch.alloc(need))
    return fail(PIMC_ERR_CUDA, "cudaMalloc displacement scratch");
  pimc_displace_record* d_rec = nullptr;
  if (records) {
    CU(cudaMallocAsync(&d_rec, sizeof(pimc_displace_record) * (size_t)e->nrep * nattempt,
                       e->stream));
    CU(cudaMemsetAsync(d_rec, 0, sizeof(pimc_displace_record) * (size_t)e->nrep * nattempt,
                       e->stream));
  }
  DisplaceParams P;
  P.sys = e->d_sys.p;
  P.state = e->d_state.p;
  P.paths = e->d_paths.p;
  P.nodecache = e->d_nodecache.p;
  P.scratch = e->d_dscratch.p;
  P.scratch_stride = sstride;
  P.nodescr_g = e->d_nodescr.p;
  P.rec = d_rec;
  P.order = e->d_order.p;
  P.next = e->d_next.p;
  P.nattempt = nattempt;
  P.nrep = e->nrep;
  P.seed = e->seed;
  for (int d = 0; d < 3; ++d) P.box[d] = box[d];
  P.nmoving = nmoving;
  P.species = species;
  P.lay = L;
  P.stage_off = stage_off;
  cudaFuncSetAttribute(displace_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemLimit);
  CU(cudaMemsetAsync(e->d_next.p, 0, sizeof(int), e->stream));
  displace_kernel<<<e->grid, dthreads, smem, e->stream>>>(P);
  e->launches++;
  CU(cudaGetLastError());
  // displaced paths: every slice's structure factors are rebuilt
  if (int rc = prefill_ewald(e, nullptr, e->nrep)) return rc;
  if (records) {
    CU(cudaMemcpyAsync(records, d_rec, sizeof(pimc_displace_record) * (size_t)e->nrep * nattempt,
                       cudaMemcpyDeviceToHost, e->stream));
    CU(cudaFreeAsync(d_rec, e->stream));
    CU(cudaStreamSynchronize(e->stream));
  }
  return PIMC_OK;
}

int pimc_virial_energy(pimc_engine* e, int nwindow, double* host_energy) {
  if (!e || e->server || nwindow < 1 || !host_energy) return fail(PIMC_ERR_INVALID, "bad argument");
  EstimatorParams P{};
  P.nwindow = nwindow;
  return run_estimator(e, kEstVirial, P, e->est_lay, host_energy);
}

int pimc_coulomb_energy(pimc_engine* e, double epsilon, double* host_energy) {
  if (!e || e->server || !(epsilon > 0) || !host_energy)
    return fail(PIMC_ERR_INVALID, "bad argument");
  EstimatorParams P{};
  P.epsilon = epsilon;
  return run_estimator(e, kEstCoulomb, P, e->est_lay, host_energy);
}

int pimc_ewald_coulomb_energy(pimc_engine* e, double epsilon, double rcut,
                              const pimc_ewald_table* est, const double* vgrid,
                              double* host_energy) {
  if (!e || e->server || !(epsilon > 0) || !(rcut > 0) || !est || !vgrid || !host_energy ||
      est->totk < 0 || (est->totk > 0 && (!est->kvec || !est->vk)))
    return fail(PIMC_ERR_INVALID, "bad argument");
  DevBuf<int> kv;
  DevBuf<double> vk, vg;
  if (kv.alloc(3 * std::max(est->totk, 1)) || vk.alloc(std::max(est->totk, 1)) || vg.alloc(1001))
    return fail(PIMC_ERR_CUDA, "cudaMalloc estimator tables");
  if (est->totk > 0) {
    CU(cudaMemcpy(kv.p, est->kvec, 3 * est->totk * sizeof(int), cudaMemcpyHostToDevice));
    CU(cudaMemcpy(vk.p, est->vk, est->totk * sizeof(double), cudaMemcpyHostToDevice));
  }
  CU(cudaMemcpy(vg.p, vgrid, 1001 * sizeof(double), cudaMemcpyHostToDevice));
  EstimatorParams P{};
  P.epsilon = epsilon;
  P.vgrid = vg.p;
  P.rcut = rcut;
  P.totk = est->totk;
  P.kvec = kv.p;
  P.vk = vk.p;
  P.one_over_2v = est->one_over_2v;
  P.self_energy = est->self_energy;
  for (int a = 0; a < 3; ++a) P.ikmax[a] = est->ikmax[a];
  const Layout L = estimator_layout(e->hsys, est->ikmax);
  const int rc = run_estimator(e, kEstCoulomb, P, L, host_energy);
  return rc;
}

int pimc_run_steps(pimc_engine* e, int nattempt, int nsteps, double* host_energy) {
  if (!e || e->server || nattempt < 0 || nsteps <= 0)
    return fail(PIMC_ERR_INVALID, "bad argument");
  if (e->graph && (e->graph_attempts != nattempt || e->graph_steps != nsteps)) {
    cudaGraphExecDestroy(e->graph);
    e->graph = nullptr;
  }
  if (!e->graph) {
    // make the buffers the graph will use before capturing it
    if (e->d_partial.n < (size_t)e->nrep * kThermoChunks &&
        e->d_partial.alloc((size_t)e->nrep * kThermoChunks))
      return fail(PIMC_ERR_CUDA, "cudaMalloc energy partials");
    if (e->d_energy.n < (size_t)nsteps * e->nrep && e->d_energy.alloc((size_t)nsteps * e->nrep))
      return fail(PIMC_ERR_CUDA, "cudaMalloc energies");
    if (!e->cap_stream) CU(cudaStreamCreateWithFlags(&e->cap_stream, cudaStreamNonBlocking));
    const long long l0 = e->launches;
    CU(cudaStreamBeginCapture(e->cap_stream, cudaStreamCaptureModeThreadLocal));
    int rc = PIMC_OK;
    for (int k = 0; k < nsteps && rc == PIMC_OK; ++k) {
      if (nattempt > 0) {
        RunParams P;
        fill_run_params(e, P, nattempt, nullptr);
        cudaMemsetAsync(e->d_next.p, 0, sizeof(int), e->cap_stream);
        section_launch(e->minb, e->grid, e->block, e->lay.total * 8, e->cap_stream, P, e->nodes);
      }
      rc = enqueue_thermo(e, e->cap_stream, k);
    }
    cudaGraph_t g = nullptr;
    const cudaError_t ce = cudaStreamEndCapture(e->cap_stream, &g);
    e->launches = l0;
    if (rc != PIMC_OK) {
      if (g) cudaGraphDestroy(g);
      return rc;
    }
    if (ce != cudaSuccess) return fail(PIMC_ERR_CUDA, cudaGetErrorString(ce));
    const cudaError_t ie = cudaGraphInstantiate(&e->graph, g, 0);
    cudaGraphDestroy(g);
    if (ie != cudaSuccess) {
      e->graph = nullptr;
      return fail(PIMC_ERR_CUDA, cudaGetErrorString(ie));
    }
    e->graph_attempts = nattempt;
    e->graph_steps = nsteps;
  }
  CU(cudaGraphLaunch(e->graph, e->stream));
  e->launches += (long long)nsteps * ((nattempt > 0 ? 1 : 0) + 2);
  if (host_energy) {
    CU(cudaMemcpyAsync(host_energy, e->d_energy.p, (size_t)nsteps * e->nrep * sizeof(double),
                       cudaMemcpyDeviceToHost, e->stream));
    CU(cudaStreamSynchronize(e->stream));
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
  // the section layout with every bead's Ewald tables and no Slater scratch
  LayoutOpts aopt;
  aopt.scratch_global = true;
  aopt.full_ewald_tables = true;
  bool lok = false;
  const Layout alay = make_layout(e->hsys, kBlock / 32, lok, aopt);
  if (!lok) return fail(PIMC_ERR_CAPACITY, "working set does not fit in shared memory");
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
  P.lay = alay;
  action_diff_kernel<<<nbatch, kBlock, P.lay.total * 8, e->stream>>>(P);
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

int pimc_fp32_peak(double* tflops) {
  if (!tflops) return fail(PIMC_ERR_INVALID, "null argument");
  int nsm = 0;
  if (int rc = device_check(nsm)) return rc;
  float* d = nullptr;
  CU(cudaMalloc(&d, sizeof(float)));
  const int iters = 16384, blocks = nsm * 8, threads = 256;
  fp32_probe_kernel<<<blocks, threads>>>(d, 16);
  cudaEvent_t a, b;
  CU(cudaEventCreate(&a));
  CU(cudaEventCreate(&b));
  float best = 1e30f;
  for (int rep = 0; rep < 5; ++rep) {
    CU(cudaEventRecord(a));
    fp32_probe_kernel<<<blocks, threads>>>(d, iters);
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

// ------------------------------------------------- launch configuration
namespace {
int apply_config(pimc_engine* e, int block, LayoutOpts opts, int ctas_cap, int minb) {
  if (minb < 1 || minb > 4) return fail(PIMC_ERR_INVALID, "register variant must be 1, 2, 3 or 4");
  bool fixed = false;
  for (const DevSys& d : e->hsys) fixed |= d.fixed_node != 0;
  // one warp per replica (block 32) only for systems without node models
  if (block != 64 && block != 128 && block != 256 && !(block == 512 && minb == 1) &&
      !(block == 32 && !fixed && minb >= 2))
    return fail(PIMC_ERR_INVALID,
                "block must be 64, 128, 256 (512 with variant 1, 32 without node models)");
  bool ok = false;
  const Layout L = make_layout(e->hsys, block / 32, ok, opts);
  if (!ok) return fail(PIMC_ERR_CAPACITY, "working set does not fit in shared memory");
  int occ = 1;
  occ = section_occupancy(minb, block, L.total * 8, e->nodes);
  occ = std::max(occ, 1);
  if (ctas_cap > 0) occ = std::min(occ, ctas_cap);
  const int grid = std::min(e->nrep, e->num_sms * occ);
  if (L.gcta > 0) {
    const size_t need = (size_t)grid * L.gcta;
    if (need > e->d_nodescr.n) {
      CU(cudaStreamSynchronize(e->stream));
      if (e->d_nodescr.alloc(need)) return fail(PIMC_ERR_CUDA, "cudaMalloc node scratch");
    }
  }
  if (e->ekstage_stride > 0 && (size_t)grid * e->ekstage_stride > e->d_ekstage.n) {
    CU(cudaStreamSynchronize(e->stream));
    if (e->d_ekstage.alloc((size_t)grid * e->ekstage_stride))
      return fail(PIMC_ERR_CUDA, "cudaMalloc structure-factor staging");
  }
  if (int rc = ensure_xstage(e, grid)) return rc;
  e->lay = L;
  e->lay_opts = opts;
  e->ctas_cap = ctas_cap;
  e->minb = minb;
  e->block = block;
  e->grid = grid;
  if (e->graph) {  // captured with the old launch shape
    cudaGraphExecDestroy(e->graph);
    e->graph = nullptr;
  }
  return PIMC_OK;
}
}  // namespace

int pimc_engine_configure(pimc_engine* e, const pimc_launch_config* cfg) {
  if (!e || !cfg) return fail(PIMC_ERR_INVALID, "bad argument");
  if (cfg->scratch_global < 0 || cfg->scratch_global > 2)
    return fail(PIMC_ERR_INVALID, "scratch_global must be 0, 1 or 2");
  if (e->server) {
    // a server's block size is fixed while it serves (a slot's sums must not
    // depend on the mix): set it before the first admission
    if (e->nactive > 0) return fail(PIMC_ERR_INVALID, "configure a server before admitting");
    for (int r = 0; r < e->nrep; ++r)
      if (e->active[r]) return fail(PIMC_ERR_INVALID, "configure a server before admitting");
    const int minb = cfg->regs_variant ? cfg->regs_variant : 2;
    if (!((cfg->block == 64 || cfg->block == 128 || cfg->block == 256) && minb >= 2 && minb <= 4) &&
        !(cfg->block == 512 && minb == 1))
      return fail(PIMC_ERR_INVALID, "block must be 64, 128, 256 (or 512 with variant 1)");
    e->block = cfg->block;
    e->minb = minb;
    e->lay_opts.scratch_global = cfg->scratch_global == 1;
    e->lay_opts.cold_global = cfg->scratch_global == 2;
    e->order_dirty = true;
    return PIMC_OK;
  }
  LayoutOpts o;
  o.scratch_global = cfg->scratch_global == 1;
  o.cold_global = cfg->scratch_global == 2;
  return apply_config(e, cfg->block, o, cfg->ctas_per_sm, cfg->regs_variant ? cfg->regs_variant : 2);
}

int pimc_engine_get_config(pimc_engine* e, pimc_launch_config* cfg) {
  if (!e || !cfg) return fail(PIMC_ERR_INVALID, "bad argument");
  cfg->block = e->block;
  cfg->scratch_global = e->lay_opts.scratch_global ? 1 : (e->lay_opts.cold_global ? 2 : 0);
  cfg->ctas_per_sm = e->ctas_cap;
  cfg->regs_variant = e->minb;
  cfg->ms = 0.f;
  return PIMC_OK;
}

int pimc_engine_autotune(pimc_engine* e, int nattempt, pimc_launch_config* best,
                         pimc_launch_config* tried, int max_tried, int* ntried) {
  if (!e || e->server || nattempt <= 0 || !best) return fail(PIMC_ERR_INVALID, "bad argument");
  // state the trials advance, kept aside and restored before each trial
  DevBuf<double> paths0, cache0;
  DevBuf<long long> ek0;
  DevBuf<DevState> state0;
  const size_t np_ = e->path_off[e->nrep];
  if (paths0.alloc(np_) || state0.alloc(e->nrep) || cache0.alloc(e->d_nodecache.n) ||
      ek0.alloc(e->d_ekcache.n))
    return fail(PIMC_ERR_CUDA, "cudaMalloc autotune backup");
  auto copy = [&](bool save) -> int {
    CU(cudaMemcpyAsync(save ? paths0.p : e->d_paths.p, save ? e->d_paths.p : paths0.p,
                       np_ * sizeof(double), cudaMemcpyDeviceToDevice, e->stream));
    CU(cudaMemcpyAsync(save ? state0.p : e->d_state.p, save ? e->d_state.p : state0.p,
                       e->nrep * sizeof(DevState), cudaMemcpyDeviceToDevice, e->stream));
    if (e->d_nodecache.n)
      CU(cudaMemcpyAsync(save ? cache0.p : e->d_nodecache.p, save ? e->d_nodecache.p : cache0.p,
                         e->d_nodecache.n * sizeof(double), cudaMemcpyDeviceToDevice, e->stream));
    if (e->d_ekcache.n)
      CU(cudaMemcpyAsync(save ? ek0.p : e->d_ekcache.p, save ? e->d_ekcache.p : ek0.p,
                         e->d_ekcache.n * sizeof(long long), cudaMemcpyDeviceToDevice, e->stream));
    return PIMC_OK;
  };
  if (int rc = copy(true)) return rc;
  const long long launches0 = e->launches;
  const int blk0 = e->block, cap0 = e->ctas_cap, minb0 = e->minb;
  const LayoutOpts opt0 = e->lay_opts;
  bool fixed = false;
  for (const DevSys& d : e->hsys) fixed |= d.fixed_node != 0;
  std::vector<pimc_launch_config> cand;
  for (int v : {2, 3, 4})
    for (int b : {32, 64, 128, 256})
      if (b > 32 || !fixed)
        for (int g = 0; g < (fixed ? 3 : 1); ++g) cand.push_back({b, g, 0, v, 0.f});
  for (int g = 0; g < (fixed ? 3 : 1); ++g) cand.push_back({512, g, 0, 1, 0.f});
  cudaEvent_t t0, t1;
  CU(cudaEventCreate(&t0));
  CU(cudaEventCreate(&t1));
  int nt = 0, ibest = -1;
  for (pimc_launch_config& c : cand) {
    LayoutOpts o;
    o.scratch_global = c.scratch_global == 1;
    o.cold_global = c.scratch_global == 2;
    if (apply_config(e, c.block, o, c.ctas_per_sm, c.regs_variant) != PIMC_OK) {
      c.ms = -1.f;  // does not fit
      continue;
    }
    float best_ms = 1e30f;
    for (int rep = 0; rep < 3; ++rep) {  // a warm-up trial, then the best of two timed ones
      if (int rc = copy(false)) return rc;
      CU(cudaEventRecord(t0, e->stream));
      if (int rc = pimc_run_sections(e, nattempt, nullptr)) return rc;
      CU(cudaEventRecord(t1, e->stream));
      CU(cudaEventSynchronize(t1));
      float ms = 0.f;
      CU(cudaEventElapsedTime(&ms, t0, t1));
      if (rep >= 1) best_ms = std::min(best_ms, ms);
    }
    c.ms = best_ms;
    if (ibest < 0 || c.ms < cand[ibest].ms) ibest = (int)(&c - &cand[0]);
  }
  // Short trials leave near-ties undecided: the three fastest are timed again
  // on three times the attempts (a warm-up and the best of two), and the
  // fastest of that decides.
  {
    std::vector<int> top;
    for (int i = 0; i < (int)cand.size(); ++i)
      if (cand[i].ms > 0) top.push_back(i);
    std::sort(top.begin(), top.end(), [&](int a, int b) { return cand[a].ms < cand[b].ms; });
    if (top.size() > 3) top.resize(3);
    float best_long = 1e30f;
    for (int i : top) {
      const pimc_launch_config& c = cand[i];
      LayoutOpts o;
      o.scratch_global = c.scratch_global == 1;
      o.cold_global = c.scratch_global == 2;
      if (apply_config(e, c.block, o, c.ctas_per_sm, c.regs_variant) != PIMC_OK) continue;
      float t = 1e30f;
      for (int rep = 0; rep < 3; ++rep) {
        if (int rc = copy(false)) return rc;
        CU(cudaEventRecord(t0, e->stream));
        if (int rc = pimc_run_sections(e, 3 * nattempt, nullptr)) return rc;
        CU(cudaEventRecord(t1, e->stream));
        CU(cudaEventSynchronize(t1));
        float ms = 0.f;
        CU(cudaEventElapsedTime(&ms, t0, t1));
        if (rep >= 1) t = std::min(t, ms);
      }
      if (t < best_long) {
        best_long = t;
        ibest = i;
      }
    }
  }
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  for (const pimc_launch_config& c : cand) {
    if (tried && nt < max_tried) tried[nt] = c;
    ++nt;
  }
  if (ntried) *ntried = nt;
  int rc;
  if (ibest >= 0) {
    // the placement the trial ran: 1 all scratch global, 2 only its cold part
    LayoutOpts o;
    o.scratch_global = cand[ibest].scratch_global == 1;
    o.cold_global = cand[ibest].scratch_global == 2;
    rc = apply_config(e, cand[ibest].block, o, cand[ibest].ctas_per_sm, cand[ibest].regs_variant);
    *best = cand[ibest];
  } else {
    rc = apply_config(e, blk0, opt0, cap0, minb0);
    pimc_engine_get_config(e, best);
  }
  if (int rc2 = copy(false)) return rc2;
  CU(cudaStreamSynchronize(e->stream));
  e->launches = launches0;  // trials are not the caller's launches
  return rc;
}

// ---------------------------------------------------------------- serving
namespace {
long long pool_alloc(pimc_engine* e, long long words) {
  for (auto it = e->free_blocks.begin(); it != e->free_blocks.end(); ++it) {
    if (it->second >= words) {
      const long long off = it->first, rest = it->second - words;
      e->free_blocks.erase(it);
      if (rest > 0) e->free_blocks[off + words] = rest;
      return off;
    }
  }
  return -1;
}
void pool_free(pimc_engine* e, long long off, long long words) {
  if (words <= 0) return;
  auto it = e->free_blocks.emplace(off, words).first;
  auto nx = std::next(it);
  if (nx != e->free_blocks.end() && it->first + it->second == nx->first) {
    it->second += nx->second;
    e->free_blocks.erase(nx);
  }
  if (it != e->free_blocks.begin()) {
    auto pv = std::prev(it);
    if (pv->first + pv->second == it->first) {
      pv->second += it->second;
      e->free_blocks.erase(it);
    }
  }
}
int refresh_order(pimc_engine* e) {
  if (!e->order_dirty) return 0;
  std::vector<std::pair<double, int>> act;
  for (int r = 0; r < e->nrep; ++r)
    if (e->active[r]) {
      const DevSys& d = e->hsys[r];
      double c = (double)d.npart * d.npart;
      for (int i = 0; i < d.nspecies; ++i)
        if (d.node_kind[i]) c += 2.0 * d.spec_count[i] * d.spec_count[i] * (d.spec_count[i] + 20);
      act.push_back({-c * ((1 << d.nlevel) + 1), r});
    }
  std::stable_sort(act.begin(), act.end());
  std::vector<int> order(act.size());
  std::vector<DevSys> live;
  for (size_t k = 0; k < act.size(); ++k) {
    order[k] = act[k].second;
    live.push_back(e->hsys[act[k].second]);
  }
  e->nactive = (int)order.size();
  if (!order.empty()) {
    // shared-memory layout and grid sized to the systems now admitted; the
    // block size stays fixed so that a slot's arithmetic never depends on the mix
    bool ok = false;
    e->lay = make_layout(live, e->block / 32, ok, e->lay_opts);
    if (!ok) return fail(PIMC_ERR_CAPACITY, "working set does not fit in shared memory");
    int occ = 1;
    occ = section_occupancy(e->minb, e->block, e->lay.total * 8);
    e->grid = std::min(e->nactive, e->num_sms * std::max(occ, 1));
    if (int rc = ensure_xstage(e, e->grid)) return rc;
    if (e->lay.gcta > 0) {
      const size_t need = (size_t)e->grid * e->lay.gcta;
      if (need > e->d_nodescr.n) {
        CU(cudaStreamSynchronize(e->stream));
        if (e->d_nodescr.alloc(need)) return fail(PIMC_ERR_CUDA, "cudaMalloc node scratch");
      }
    }
    CU(cudaMemcpyAsync(e->d_order.p, order.data(), order.size() * sizeof(int),
                       cudaMemcpyHostToDevice, e->stream));
    CU(cudaStreamSynchronize(e->stream));
  }
  e->order_dirty = false;
  return 0;
}
}  // namespace

int pimc_server_create(const pimc_server_config* cfg, uint64_t seed, int precision,
                       pimc_engine** out) {
  if (!cfg || !out || cfg->slots <= 0 || cfg->hbm_bytes < 1024 || cfg->max_npart <= 0 ||
      cfg->max_level < 1 || cfg->max_level > PIMC_MAX_LEVEL || cfg->max_nslice <= 0 ||
      cfg->max_node_count < 0 || cfg->max_node_count > PIMC_MAX_NODE_PARTICLES)
    return fail(PIMC_ERR_INVALID, "bad server configuration");
  *out = nullptr;
  int nsm = 0;
  if (int rc = device_check(nsm)) return rc;
  pimc_engine* e = new pimc_engine();
  e->server = true;
  e->scfg = *cfg;
  e->nrep = cfg->slots;
  e->seed = seed;
  e->precision = precision;
  e->num_sms = nsm;
  e->hsys.assign(cfg->slots, DevSys());
  e->hdesc.resize(cfg->slots);
  e->active.assign(cfg->slots, 0);
  e->slot_path.assign(cfg->slots, -1);
  e->slot_cache.assign(cfg->slots, -1);
  e->slot_words.assign(cfg->slots, 0);
  e->slot_attempts.assign(cfg->slots, 1);
  e->path_off.assign(cfg->slots + 1, 0);
  // layout for the largest admissible system
  DevSys mx;
  memset(&mx, 0, sizeof(mx));
  mx.npart = cfg->max_npart;
  mx.nlevel = cfg->max_level;
  mx.nsec = (1 << cfg->max_level) + 1;
  mx.nslice = cfg->max_nslice;
  mx.ns_max = std::max(1, cfg->max_node_count);
  mx.fixed_node = cfg->max_node_count > 0;
  mx.nspecies = 2;
  mx.node_kind[0] = mx.fixed_node ? PIMC_NODES_SHO : 0;
  std::vector<DevSys> one(1, mx);
  e->block = kBlock;
  bool ok = false;
  const Layout biggest = make_layout(one, e->block / 32, ok);
  if (!ok) {
    delete e;
    return fail(PIMC_ERR_CAPACITY, "largest system does not fit in shared memory");
  }
  set_smem_caps();
  e->lay = biggest;
  e->grid = std::min(cfg->slots, nsm);
  if (precision == PIMC_PREC_MIXED && mx.fixed_node)
    e->xstage_cta = (long long)mx.nsec * (mx.ns_max * mx.ns_max + 2);
  const long long words = (long long)(cfg->hbm_bytes / sizeof(double));
  if (e->d_pool.alloc(words) || e->d_sys.alloc(cfg->slots) || e->d_state.alloc(cfg->slots) ||
      e->d_order.alloc(cfg->slots) || e->d_next.alloc(1) || e->d_slot_attempts.alloc(cfg->slots) || e->d_ugrid.alloc(1 << 22) ||
      e->d_ugrid32.alloc(1 << 22)) {
    delete e;
    return fail(PIMC_ERR_CUDA, "cudaMalloc server pool");
  }
  e->free_blocks[0] = words;
  *out = e;
  return PIMC_OK;
}

int pimc_server_admit(pimc_engine* e, const pimc_system* sys, const pimc_pair_table* tables,
                      int ntables, const double* host_path, uint32_t stream_id,
                      int round_attempts, int* slot) {
  if (!e || !e->server || !sys || !host_path || !slot || (ntables > 0 && !tables) ||
      round_attempts <= 0)
    return fail(PIMC_ERR_INVALID, "bad argument");
  if (int rc = validate(*sys)) return rc == PIMC_ERR_CAPACITY ? PIMC_ERR_INVALID : rc;
  if (sys->ewald) return fail(PIMC_ERR_INVALID, "the server takes no Ewald systems");
  DevSys d;
  fill_sys(*sys, d);
  if (d.npart > e->scfg.max_npart || d.nlevel > e->scfg.max_level ||
      d.nslice > e->scfg.max_nslice || (d.fixed_node && d.ns_max > e->scfg.max_node_count))
    return fail(PIMC_ERR_INVALID, "system larger than the server's maxima");
  int r = -1;
  for (int k = 0; k < e->nrep; ++k)
    if (!e->active[k]) {
      r = k;
      break;
    }
  if (r < 0) return fail(PIMC_ERR_CAPACITY, "no free slot");
  const long long pw = 3LL * sys->nslice * sys->npart;
  const bool cache = d.fixed_node && (1 << d.nlevel) < d.nslice / 2;
  d.mixed = e->precision == PIMC_PREC_MIXED;
  d.nc_stride = cache_entry_doubles(d);
  const long long cw = cache ? (long long)d.nspecies * d.nslice * d.nc_stride : 0;
  const long long po = pool_alloc(e, pw + cw);
  if (po < 0) return fail(PIMC_ERR_CAPACITY, "device pool full");
  // pair tables: one device copy per distinct host table
  if (sys->coulomb) {
    if (ntables > kMaxTables) {
      pool_free(e, po, pw + cw);
      return fail(PIMC_ERR_CAPACITY, "too many pair tables");
    }
    for (int k = 0; k < ntables; ++k) {
      const pimc_pair_table& t = tables[k];
      if (t.species1 < 0 || t.species1 >= sys->nspecies || t.species2 < 0 ||
          t.species2 >= sys->nspecies || t.ngpts < 2 || t.norder < 0 || !t.ugrid) {
        pool_free(e, po, pw + cw);
        return fail(PIMC_ERR_INVALID, "bad pair table");
      }
      const size_t words = (size_t)t.ngpts * 2 * (t.norder + 1);
      size_t toff = (size_t)-1;
      auto range = e->table_dev.equal_range(t.ugrid);
      for (auto it = range.first; it != range.second; ++it)
        if (it->second.second.size() == words &&
            std::equal(t.ugrid, t.ugrid + words, it->second.second.begin()))
          toff = it->second.first;
      if (toff == (size_t)-1) {
        if (e->table_used + words > e->d_ugrid.n) {
          pool_free(e, po, pw + cw);
          return fail(PIMC_ERR_INVALID, "server table pool full (distinct pair tables exceed 32 MiB)");
        }
        toff = e->table_used;
        std::vector<float> f(t.ugrid, t.ugrid + words);
        CU(cudaMemcpy(e->d_ugrid.p + toff, t.ugrid, words * 8, cudaMemcpyHostToDevice));
        CU(cudaMemcpy(e->d_ugrid32.p + toff, f.data(), words * 4, cudaMemcpyHostToDevice));
        e->table_used += words;
        e->table_dev.emplace(t.ugrid, std::make_pair(toff, std::vector<double>(t.ugrid, t.ugrid + words)));
      }
      DevTable& dt = d.tab[k];
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
      dt.ugrid = e->d_ugrid.p + toff;
      dt.ugrid32 = e->d_ugrid32.p + toff;
    }
    d.ntab = ntables;
  }
  d.mixed = e->precision == PIMC_PREC_MIXED;
  d.stream_id = stream_id;
  d.path_offset = po;
  d.nc_offset = cache ? po + pw : -1;
  d.inv_offset = e->lay.gcta > 0 ? 0 : -1;
  e->hsys[r] = d;
  e->hdesc[r] = *sys;
  e->slot_path[r] = po;
  e->slot_words[r] = pw + cw;
  e->active[r] = 1;
  e->order_dirty = true;
  DevState st;
  memset(&st, 0, sizeof(st));
  for (int k = 0; k < kMaxSpecies; ++k) st.node_scale[k] = 1.0;
  for (long long i = 0; i < pw; ++i)  // the admission's counterpart of path_scan_kernel
    if (!std::isfinite(host_path[i])) {
      st.status |= PIMC_STATUS_NONFINITE;
      break;
    }
  CU(cudaMemcpyAsync(e->d_sys.p + r, &e->hsys[r], sizeof(DevSys), cudaMemcpyHostToDevice,
                     e->stream));
  CU(cudaMemcpyAsync(e->d_state.p + r, &st, sizeof(DevState), cudaMemcpyHostToDevice, e->stream));
  e->slot_attempts[r] = round_attempts;
  if (cw) e->prefill_pending.push_back(r);
  CU(cudaMemcpyAsync(e->d_slot_attempts.p + r, &e->slot_attempts[r], sizeof(int),
                     cudaMemcpyHostToDevice, e->stream));
  CU(cudaMemcpyAsync(e->d_pool.p + po, host_path, pw * sizeof(double), cudaMemcpyHostToDevice,
                     e->stream));
  if (cw) CU(cudaMemsetAsync(e->d_pool.p + po + pw, 0xff, cw * sizeof(double), e->stream));
  CU(cudaStreamSynchronize(e->stream));  // the host copies above are from caller memory
  *slot = r;
  return PIMC_OK;
}

int pimc_server_release(pimc_engine* e, int slot) {
  if (!e || !e->server || slot < 0 || slot >= e->nrep || !e->active[slot])
    return fail(PIMC_ERR_INVALID, "bad slot");
  CU(cudaStreamSynchronize(e->stream));  // no launch may still use the slot's memory
  pool_free(e, e->slot_path[slot], e->slot_words[slot]);
  e->active[slot] = 0;
  e->order_dirty = true;
  return PIMC_OK;
}

int pimc_server_run(pimc_engine* e) {
  if (!e || !e->server) return fail(PIMC_ERR_INVALID, "bad argument");
  if (int rc = refresh_order(e)) return rc;
  if (e->nactive == 0) return PIMC_OK;
  if (!e->prefill_pending.empty()) {
    // newly admitted simulations: their Slater caches, filled in parallel
    std::vector<int> live;
    for (int r : e->prefill_pending)
      if (e->active[r]) live.push_back(r);
    e->prefill_pending.clear();
    if (!live.empty()) {
      if (e->d_prefill.n < live.size() && e->d_prefill.alloc(std::max<size_t>(live.size(), 64)))
        return fail(PIMC_ERR_CUDA, "cudaMalloc prefill list");
      CU(cudaMemcpyAsync(e->d_prefill.p, live.data(), live.size() * sizeof(int),
                         cudaMemcpyHostToDevice, e->stream));
      if (int rc = prefill_cache(e, e->d_pool.p, e->d_prefill.p, (int)live.size())) return rc;
      CU(cudaStreamSynchronize(e->stream));  // the host list is reused next round
    }
  }
  const int nattempt = 0;
  RunParams P;
  P.sys = e->d_sys.p;
  P.state = e->d_state.p;
  P.paths = e->d_pool.p;
  P.nodescr_g = e->d_nodescr.p;
  P.nodecache = e->d_pool.p;
  P.ekcache = nullptr;  // servers take no Ewald systems
  P.ekstage = nullptr;
  P.ekstage_stride = 0;
  P.xstage = e->xstage_cta > 0 ? e->d_xstage.p : nullptr;
  P.xstage_cta = e->xstage_cta;
  P.rec = nullptr;
  P.order = e->d_order.p;
  P.next = e->d_next.p;
  P.nattempt = nattempt;
  P.nattempt_r = e->d_slot_attempts.p;
  P.nrep = e->nactive;
  P.seed = e->seed;
  P.lay = e->lay;
  CU(cudaMemsetAsync(e->d_next.p, 0, sizeof(int), e->stream));
  CU(section_launch(e->minb, e->grid, e->block, e->lay.total * 8, e->stream, P));
  e->launches++;
  return PIMC_OK;
}

}  // extern "C"

namespace {
// ThermoEnergyEstimator's value for the listed slots (host list) into out[k].
int server_energy(pimc_engine* e, const std::vector<int>& slots, double* out) {
  const int n = (int)slots.size();
  if (n == 0) return PIMC_OK;
  // a fixed chunk count: each slot's sum is grouped the same way whatever the mix
  const int nchunk = 64;
  double* d_part = nullptr;
  int* d_idx = nullptr;
  CU(cudaMallocAsync(&d_part, sizeof(double) * (size_t)n * nchunk, e->stream));
  CU(cudaMallocAsync(&d_idx, sizeof(int) * (size_t)n, e->stream));
  CU(cudaMemcpyAsync(d_idx, slots.data(), sizeof(int) * (size_t)n, cudaMemcpyHostToDevice,
                     e->stream));
  ThermoParams P;
  P.sys = e->d_sys.p;
  P.index = d_idx;
  P.paths = e->d_pool.p;
  P.ekcache = nullptr;  // servers take no Ewald systems
  P.partial = d_part;
  P.nchunk = nchunk;
  P.nrep = n;
  P.lay = e->lay;
  thermo_kernel<<<dim3(nchunk, n), kBlock, e->lay.total * 8, e->stream>>>(P);
  e->launches++;
  CU(cudaGetLastError());
  std::vector<double> part((size_t)n * nchunk);
  CU(cudaMemcpyAsync(part.data(), d_part, part.size() * 8, cudaMemcpyDeviceToHost, e->stream));
  CU(cudaFreeAsync(d_part, e->stream));
  CU(cudaFreeAsync(d_idx, e->stream));
  CU(cudaStreamSynchronize(e->stream));
  for (int k = 0; k < n; ++k) {
    double s = 0;
    for (int c = 0; c < nchunk; ++c) s += part[(size_t)k * nchunk + c];
    out[k] = s / e->hsys[slots[k]].nslice;
  }
  return PIMC_OK;
}
}  // namespace

extern "C" {

int pimc_server_energy(pimc_engine* e, double* energy) {
  if (!e || !e->server || !energy) return fail(PIMC_ERR_INVALID, "bad argument");
  if (int rc = refresh_order(e)) return rc;
  for (int r = 0; r < e->nrep; ++r) energy[r] = std::nan("");
  std::vector<int> slots;
  for (int r = 0; r < e->nrep; ++r)
    if (e->active[r]) slots.push_back(r);
  std::vector<double> out(slots.size());
  if (int rc = server_energy(e, slots, out.data())) return rc;
  for (size_t k = 0; k < slots.size(); ++k) energy[slots[k]] = out[k];
  return PIMC_OK;
}

int pimc_server_energy_slots(pimc_engine* e, const int* slots, int nslot, double* energy) {
  if (!e || !e->server || nslot < 0 || (nslot > 0 && (!slots || !energy)))
    return fail(PIMC_ERR_INVALID, "bad argument");
  for (int k = 0; k < nslot; ++k)
    if (slots[k] < 0 || slots[k] >= e->nrep || !e->active[slots[k]])
      return fail(PIMC_ERR_INVALID, "slot not in use");
  if (int rc = refresh_order(e)) return rc;
  return server_energy(e, std::vector<int>(slots, slots + nslot), energy);
}

int pimc_server_download_path(pimc_engine* e, int slot, double* host_xyz) {
  if (!e || !e->server || slot < 0 || slot >= e->nrep || !e->active[slot] || !host_xyz)
    return fail(PIMC_ERR_INVALID, "bad slot");
  const long long pw = 3LL * e->hdesc[slot].nslice * e->hdesc[slot].npart;
  CU(cudaMemcpyAsync(host_xyz, e->d_pool.p + e->slot_path[slot], pw * sizeof(double),
                     cudaMemcpyDeviceToHost, e->stream));
  CU(cudaStreamSynchronize(e->stream));
  return PIMC_OK;
}

int pimc_server_pool(pimc_engine* e, size_t* used, size_t* largest_free) {
  if (!e || !e->server) return fail(PIMC_ERR_INVALID, "not a server");
  long long fr = 0, big = 0;
  for (auto& b : e->free_blocks) {
    fr += b.second;
    big = std::max(big, b.second);
  }
  if (used) *used = (size_t)(e->d_pool.n - fr) * sizeof(double);
  if (largest_free) *largest_free = (size_t)big * sizeof(double);
  return PIMC_OK;
}

// Allocation-free node evaluation.  The device address of the static scratch
// array is looked up once per device (cudaGetSymbolAddress, with that device
// current) on the first call made on it, and cached in an atomic slot per
// device, so host threads calling concurrently see either no address or the
// whole one (two first calls racing both look it up and store the same value).
// The cache outlives a context: after cudaDeviceReset the address is stale, and
// resetting a device between calls is not supported.
namespace {
constexpr int kMaxDevices = 64;
std::atomic<double*> g_noalloc_addr[kMaxDevices];
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
  double* scratch = g_noalloc_addr[dev].load(std::memory_order_acquire);
  if (!scratch) {
    void* p = nullptr;
    CU(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    scratch = (double*)p;
    g_noalloc_addr[dev].store(scratch, std::memory_order_release);
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
  P.scratch = scratch;
  const int grid = nbatch < kNoAllocSlots ? nbatch : kNoAllocSlots;
  const size_t smem = 6 * (size_t)sys->npart * sizeof(double);
  if (smem > 48 * 1024) return fail(PIMC_ERR_CAPACITY, "npart beyond 1024");
  node_eval_noalloc_kernel<<<grid, 32, smem, (cudaStream_t)stream>>>(P);
  CU(cudaGetLastError());
  return PIMC_OK;
}

}  // extern "C"
