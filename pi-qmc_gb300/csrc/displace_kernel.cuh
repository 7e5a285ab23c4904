// Rigid displacement of whole particle paths: DisplaceMoveSampler::run/tryMove
// (src/advancer/DisplaceMoveSampler.cc:63-224) and, for fixed-node systems,
// DoubleDisplaceMoveSampler (src/advancer/DoubleDisplaceMoveSampler.cc:40-128),
// with a UniformMover (src/advancer/UniformMover.cc:25-42) and the actions'
// displacement differences: SHOAction (src/action/SHOAction.cc:107-143),
// PairAction (src/action/PairAction.cc:362-500), CoulombAction's Ewald term
// (src/action/CoulombAction.cc:123-146) and FixedNodeAction
// (src/fixednode/FixedNodeAction.cc:133-248).  SpringAction and PrimSHOAction
// contribute nothing (pi-qmc's base-class default).  One CTA per replica; the
// path is read and shifted in place in HBM.
#pragma once
#include "entry_kernels.cuh"

namespace pimc {

constexpr int kMaxMoving = 4;

struct DisplaceParams {
  const DevSys* sys;
  DevState* state;
  double* paths;
  double* nodecache;
  double* scratch;         // per CTA: node dets and distances of the new and old pairs
  long long scratch_stride;  // doubles per CTA
  double* nodescr_g;       // per-warp Slater scratch when it is not in shared memory
  pimc_displace_record* rec;  // [nrep][nattempt] or null
  const int* order;
  int* next;
  int nattempt;
  int nrep;
  uint64_t seed;
  double box[3];
  int nmoving;
  int species;  // -1: any particle
  Layout lay;
  int stage_off;  // doubles into shared memory: per-group slice-pair staging (6 npart each)
};

// Bead b of particle p at slice t (wrapping the slice index).
__device__ __forceinline__ const double* bead_at(const double* path, int np, int M, int p, int t) {
  t = t < 0 ? t + M : (t >= M ? t - M : t);
  return path + ((size_t)t * np + p) * 3;
}

__global__ void __launch_bounds__(kBlock) displace_kernel(DisplaceParams P) {
  extern __shared__ double smem[];
  __shared__ DevSys S;
  __shared__ int mov[kMaxMoving];
  __shared__ double dsp[kMaxMoving][3];
  __shared__ int epoch[kMaxSpecies];
  __shared__ double scale[kMaxSpecies];
  __shared__ uint32_t status;
  __shared__ long long nacc;
  __shared__ int rnext, flag;
  __shared__ double node_total;
  __shared__ Smem M_;  // carved pointers, shared so that callees read them from shared memory
  for (;;) {
    if (threadIdx.x == 0) {
      const int k = atomicAdd(P.next, 1);
      rnext = (k < P.nrep) ? P.order[k] : -1;
    }
    __syncthreads();
    const int r = rnext;
    if (r < 0) break;
    {
      const int* src = (const int*)(P.sys + r);
      int* dst = (int*)&S;
      for (int i = threadIdx.x; i < (int)(sizeof(DevSys) / sizeof(int)); i += blockDim.x)
        dst[i] = src[i];
    }
    if (threadIdx.x == 0) {
      M_ = carve(smem, P.lay, P.sys[r], P.nodescr_g);
      status = P.state[r].status;
      nacc = 0;
      for (int k = 0; k < kMaxSpecies; ++k) {
        epoch[k] = P.state[r].epoch[k];
        scale[k] = P.state[r].node_scale[k];
      }
    }
    __syncthreads();
    const DevSys& s = S;
    const Smem& m = M_;
    double* path = P.paths + s.path_offset;
    double* cache = (P.nodecache && s.nc_offset >= 0) ? P.nodecache + s.nc_offset : nullptr;
    double* scr = P.scratch + (size_t)blockIdx.x * P.scratch_stride;
    const int np = s.npart, M = s.nslice, nmov = P.nmoving;
    const int half = M / 2;
    const bool dbl = s.fixed_node != 0;
    const int i2 = dbl ? half - 1 : M - 1;
    const uint32_t att0 = P.state[r].attempt;
    for (int i = threadIdx.x; i < np; i += blockDim.x) m.qpart[i] = s.charge[species_of(s, i)];
    for (int a = 0; a < P.nattempt; ++a) {
      const uint32_t att = att0 + (uint32_t)a;
      // ---- particles and displacement (thread 0, pi-qmc's random-number order)
      if (threadIdx.x == 0) {
        uint32_t ui = 0;
        for (int im = 0; im < nmov;) {
          int i;
          const double u = stream_uniform(P.seed, s.stream_id, att, ui++);
          if (P.species < 0) {
            i = (int)(np * u);
            if (i == np) continue;
          } else {
            const int nsp = s.spec_count[P.species], f = s.spec_first[P.species];
            i = (int)(nsp * u + f);
            if (i == nsp + f) i = nsp + f - 1;
          }
          bool dup = false;
          for (int jm = 0; jm < im; ++jm) dup |= mov[jm] == i;
          if (!dup) mov[im++] = i;
        }
        for (int k = 0; k < nmov; ++k)
          for (int d = 0; d < 3; ++d) dsp[k][d] = stream_uniform(P.seed, s.stream_id, att, ui++);
        for (int k = 0; k < nmov; ++k)
          for (int d = 0; d < 3; ++d) {
            dsp[k][d] -= 0.5;
            dsp[k][d] *= P.box[d];
          }
        m.ictl[C_IPART] = (int)ui;  // index of the Metropolis uniform
        flag = 0;
        node_total = 0.0;
      }
      __syncthreads();
      // ---- Action differences over the slice ranges [0, i2] (and [half, half + i2])
      const int nrange = dbl ? 2 : 1;
      const int len = i2 + 1;
      double part = 0.0;
      // SHOAction: moving slots up to the first particle outside the species
      for (int sp = 0; sp < s.nspecies; ++sp) {
        const double om = s.sho_omega[sp];
        if (!(om > 0)) continue;
        int mstop = 0;
        while (mstop < nmov && mov[mstop] >= s.spec_first[sp] &&
               mov[mstop] < s.spec_first[sp] + s.spec_count[sp])
          ++mstop;
        const double mw = s.mass[sp] * om, ch = s.sho_cosh0[sp], div1 = 0.5 * s.sho_csch[sp];
        for (int it = threadIdx.x; it < mstop * nrange * len; it += blockDim.x) {
          const int k = it / (nrange * len), rest = it % (nrange * len);
          const int t = (rest / len) * half + rest % len;
          const int ip = mov[k];
          const double* b1 = bead_at(path, np, M, ip, t);
          const double* b0 = bead_at(path, np, M, ip, t - 1);
          double r1[3] = {b1[0], b1[1], b1[2]}, r0[3] = {b0[0], b0[1], b0[2]};
          double v = -mw * ((dot3(r1[0], r1[1], r1[2], r1[0], r1[1], r1[2]) +
                             dot3(r0[0], r0[1], r0[2], r0[0], r0[1], r0[2])) * ch -
                            2.0 * dot3(r0[0], r0[1], r0[2], r1[0], r1[1], r1[2])) * div1;
          for (int d = 0; d < 3; ++d) {
            r1[d] += dsp[k][d];
            r0[d] += dsp[k][d];
          }
          v += mw * ((dot3(r1[0], r1[1], r1[2], r1[0], r1[1], r1[2]) +
                      dot3(r0[0], r0[1], r0[2], r0[0], r0[1], r0[2])) * ch -
                     2.0 * dot3(r0[0], r0[1], r0[2], r1[0], r1[1], r1[2])) * div1;
          part += v;
        }
      }
      // PairAction: items (moving slot, partner, slice)
      if (s.coulomb) {
        for (int ti = 0; ti < s.ntab; ++ti) {
          const DevTable& tb = s.tab[ti];
          const int items = nmov * np * nrange * len;
          for (int it = threadIdx.x; it < items; it += blockDim.x) {
            const int im = it / (np * nrange * len);
            int rest = it % (np * nrange * len);
            const int j = rest / (nrange * len);
            rest %= nrange * len;
            const int rg = rest / len, tl = rest % len;
            const int t = rg * half + tl, tfirst = rg * half;
            const int i = mov[im];
            bool in1 = i >= tb.ifirst1 && i < tb.ifirst1 + tb.npart1;
            bool in2 = i >= tb.ifirst2 && i < tb.ifirst2 + tb.npart2;
            if (!in1 && !in2) continue;
            const int jb = in1 ? tb.ifirst2 : tb.ifirst1, jn = in1 ? tb.npart2 : tb.npart1;
            if (j < jb || j >= jb + jn) continue;
            int jm = -1;
            for (int k = 0; k < nmov; ++k)
              if (mov[k] == j) {
                jm = k;
                break;
              }
            if (jm >= 0 && i <= j) continue;
            const double* bi = bead_at(path, np, M, i, t);
            const double* bj = bead_at(path, np, M, j, t);
            const double* pi = bead_at(path, np, M, i, t - 1);
            const double* pj = bead_at(path, np, M, j, t - 1);
            const double di[3] = {dsp[im][0], dsp[im][1], dsp[im][2]};
            double djx = 0, djy = 0, djz = 0;
            if (jm >= 0) {
              djx = dsp[jm][0];
              djy = dsp[jm][1];
              djz = dsp[jm][2];
            }
            // previous (moving) delta: pbc(old delta) + shift at the range's
            // first slice, the previous slice's moving delta otherwise
            double ox = pi[0] - pj[0], oy = pi[1] - pj[1], oz = pi[2] - pj[2];
            pbc(s, ox, oy, oz);
            double px, py, pz;
            if (t == tfirst) {
              px = ox + di[0];
              py = oy + di[1];
              pz = oz + di[2];
              if (jm >= 0) {
                px -= djx;
                py -= djy;
                pz -= djz;
              }
            } else {
              px = pi[0] + di[0] - pj[0];
              py = pi[1] + di[1] - pj[1];
              pz = pi[2] + di[2] - pj[2];
              if (jm >= 0) {
                px -= djx;
                py -= djy;
                pz -= djz;
              }
            }
            pbc(s, px, py, pz);
            double nx = bi[0] + di[0] - bj[0], ny = bi[1] + di[1] - bj[1], nz = bi[2] + di[2] - bj[2];
            if (jm >= 0) {
              nx -= djx;
              ny -= djy;
              nz -= djz;
            }
            pbc(s, nx, ny, nz);
            double cx = bi[0] - bj[0], cy = bi[1] - bj[1], cz = bi[2] - bj[2];
            pbc(s, cx, cy, cz);
            double v = 0.0;
            for (int pass = 0; pass < 2; ++pass) {
              const double ax = pass ? cx : nx, ay = pass ? cy : ny, az = pass ? cz : nz;
              const double bx = pass ? ox : px, by = pass ? oy : py, bz = pass ? oz : pz;
              const double rr = sqrt(dot3(ax, ay, az, ax, ay, az));
              const double rp = sqrt(dot3(bx, by, bz, bx, by, bz));
              const double q = 0.5 * (rr + rp);
              double act;
              if (tb.norder > 0) {
                const double sx = ax - bx, sy = ay - by, sz = az - bz;
                act = tab_uk0(tb, q, dot3(sx, sy, sz, sx, sy, sz) / (q * q));
              } else {
                act = tab_u00(tb, q);
              }
              v += pass ? -act : act;
            }
            part += v;
          }
        }
      }
      double ds = block_sum(part, m.red);
      // CoulombAction's long-range term on every slice of the ranges
      if (s.coulomb && s.ewald) {
        double lr = 0.0;
        for (int rg = 0; rg < nrange; ++rg)
          for (int tl = 0; tl < len; ++tl) {
            const int t = rg * half + tl;
            __syncthreads();
            for (int i = threadIdx.x; i < np; i += blockDim.x) {
              const double* b = path + ((size_t)t * np + i) * 3;
              m.s1x[i] = b[0];
              m.s1y[i] = b[1];
              m.s1z[i] = b[2];
              double x = b[0], y = b[1], z = b[2];
              for (int k = 0; k < nmov; ++k)
                if (mov[k] == i) {
                  x += dsp[k][0];
                  y += dsp[k][1];
                  z += dsp[k][2];
                  pbc(s, x, y, z);
                }
              m.s1x[np + i] = x;
              m.s1y[np + i] = y;
              m.s1z[np + i] = z;
            }
            __syncthreads();
            const double eold = ewald_slice_energy(s, m, 0);
            const double enew = ewald_slice_energy(s, m, 1);
            lr += -(eold * s.tau / s.epsilon) + enew * s.tau / s.epsilon;
          }
        ds += lr;
      }
      // ---- FixedNodeAction per node species holding a moving particle
      double dsn = 0.0;
      if (dbl) {
        const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
        const int nsm = s.ns_max;
        double* ndet = scr;                       // [half] new determinants
        double* ndist = ndet + half;              // [half][2][nsm]
        double* odist = ndist + (size_t)half * 2 * nsm;  // [half][2][nsm]
        for (int sp = 0; sp < s.nspecies; ++sp) {
          if (!s.node_kind[sp]) continue;
          bool any = false;
          for (int k = 0; k < nmov; ++k)
            any |= mov[k] >= s.spec_first[sp] && mov[k] < s.spec_first[sp] + s.spec_count[sp];
          if (!any) continue;
          const int n = s.spec_count[sp], f = s.spec_first[sp];
          const bool sho = s.node_kind[sp] == PIMC_NODES_SHO;
          const int W = node_group_width(n), G = 32 / W, g = lane / W, gl = lane & (W - 1);
          double* gscr = group_scr(m, warp, g, n, !sho);
          double* gcold = group_cold(m, warp, g, n, !sho);
          double* st = smem + P.stage_off + (size_t)(warp * G + g) * 6 * n;  // [2][3][n]
          if (threadIdx.x == 0) m.ictl[C_FLAG] = 0;
          __syncthreads();
          for (int pass = 0; pass < 2; ++pass) {  // 0: new positions, 1: old
            for (int base = warp * G; base < half; base += nwarps * G) {
              const int task = base + g;
              const bool act = task < half;
              const int t = act ? task : base;
              double* e = (pass == 1 && cache) ? cache_entry(s, cache, sp, t) : nullptr;
              const bool hit = e && e[0] == (double)epoch[sp];
              // stage this species' beads of slices t and t + M/2 (shifted on the new pass)
              for (int p = gl; p < n; p += W) {
                for (int side = 0; side < 2; ++side) {
                  const double* b = path + ((size_t)(t + side * half) * np + f + p) * 3;
                  double x = b[0], y = b[1], z = b[2];
                  if (pass == 0)
                    for (int k = 0; k < nmov; ++k)
                      if (mov[k] == f + p) {
                        x += dsp[k][0];
                        y += dsp[k][1];
                        z += dsp[k][2];
                        pbc(s, x, y, z);
                      }
                  st[(side * 3 + 0) * n + p] = x;
                  st[(side * 3 + 1) * n + p] = y;
                  st[(side * 3 + 2) * n + p] = z;
                }
              }
              __syncwarp();
              double* d1 = (pass == 0 ? ndist : odist) + (size_t)t * 2 * nsm;
              double* d2 = d1 + nsm;
              // every group of the warp evaluates (the shuffles span the warp);
              // a group whose old pair is cached stores nothing and copies the
              // cached distances instead (bit-identical values)
              {
                // node_eval_group reads particle f + p: views offset so that it
                // lands on staged entry p
                SliceView v1{st - f, st + n - f, st + 2 * n - f, n, 0, -1, 0, 0, 0};
                SliceView v2{st + 3 * n - f, st + 4 * n - f, st + 5 * n - f, n, 0, -1, 0, 0, 0};
                double det = 0;
                int err = 0;
                const bool store = act && !hit;
                node_eval_dispatch(W, s, sp, v1, v2, scale[sp], gscr, 1, nullptr, -1, store, det,
                                   err, d1, d2, nullptr, 0xffffffffu, gcold);
                if (store && gl == 0) {
                  if (pass == 0) ndet[t] = det;
                  if (err) atomicOr(&m.ictl[C_FLAG], 1);
                }
              }
              __syncwarp();
              if (act && hit)
                for (int p = gl; p < n; p += W) {
                  d1[p] = e[2 + p];
                  d2[p] = e[2 + n + p];
                }
              __syncwarp();
            }
            __syncthreads();
            if (pass == 0) {
              // a singular matrix or a sign change against the first slice rejects
              if (threadIdx.x == 0) {
                bool bad = m.ictl[C_FLAG] != 0;
                for (int t = 1; t < half && !bad; ++t) bad = ndet[t] * ndet[0] < 0.0;
                if (bad) flag = 1;
              }
              __syncthreads();
              if (flag) break;
            } else if (m.ictl[C_FLAG]) {
              if (threadIdx.x == 0) flag = 1;
            }
            __syncthreads();
          }
          if (flag) break;
          // nodal action: -sum log(new) + sum log(old) over consecutive pairs
          double np_part = 0.0;
          for (int it = threadIdx.x; it < (half - 1) * n; it += blockDim.x) {
            const int t = 1 + it / n, p = it % n;
            const double* a1 = ndist + (size_t)t * 2 * nsm;
            const double* a0 = ndist + (size_t)(t - 1) * 2 * nsm;
            const double* b1 = odist + (size_t)t * 2 * nsm;
            const double* b0 = odist + (size_t)(t - 1) * 2 * nsm;
            np_part -= log((1 - exp(-a1[p] * a0[p])) * (1 - exp(-a1[nsm + p] * a0[nsm + p])));
            np_part += log((1 - exp(-b1[p] * b0[p])) * (1 - exp(-b1[nsm + p] * b0[nsm + p])));
          }
          const double tot = block_sum(np_part, m.red);
          if (threadIdx.x == 0) node_total += tot;
          __syncthreads();
        }
        dsn = flag ? 2e100 : node_total;
      }
      // ---- Metropolis test and the shift of the accepted paths
      if (threadIdx.x == 0) {
        const double total = ds + dsn;
        const double u = stream_uniform(P.seed, s.stream_id, att, (uint32_t)m.ictl[C_IPART]);
        const bool acc = !(u > exp(-total + 0.0));
        m.ictl[C_REJECT] = acc ? 0 : 1;
        if (!isfinite(ds)) status |= PIMC_STATUS_NONFINITE;
        if (acc) ++nacc;
        if (P.rec) {
          pimc_displace_record* rc = P.rec + (size_t)r * P.nattempt + a;
          for (int k = 0; k < kMaxMoving; ++k) {
            rc->ipart[k] = k < nmov ? mov[k] : -1;
            for (int d = 0; d < 3; ++d) rc->disp[k][d] = k < nmov ? dsp[k][d] : 0.0;
          }
          rc->ds = ds;
          rc->ds_node = dbl ? dsn : 0.0;
          rc->accepted = acc ? 1 : 0;
        }
        if (acc && dbl)
          for (int sp = 0; sp < s.nspecies; ++sp)
            for (int k = 0; k < nmov; ++k)
              if (mov[k] >= s.spec_first[sp] && mov[k] < s.spec_first[sp] + s.spec_count[sp]) {
                epoch[sp] += 1;  // every slice pair of the species changed
                break;
              }
      }
      __syncthreads();
      if (m.ictl[C_REJECT] == 0 && dbl && cache) {
        // the species' cached element matrices are stale in rows and columns
        for (int sp = 0; sp < s.nspecies; ++sp) {
          bool any = false;
          for (int k = 0; k < nmov; ++k)
            any |= mov[k] >= s.spec_first[sp] && mov[k] < s.spec_first[sp] + s.spec_count[sp];
          if (!any || !s.node_kind[sp]) continue;
          const int ms = cache_mask_slot(s, sp);
          for (int t = threadIdx.x; t < M; t += blockDim.x)
            cache_entry(s, cache, sp, t)[ms] = __longlong_as_double(-1ll);
        }
      }
      if (m.ictl[C_REJECT] == 0) {
        for (int it = threadIdx.x; it < nmov * M; it += blockDim.x) {
          const int k = it / M, t = it % M;
          double* b = path + ((size_t)t * np + mov[k]) * 3;
          double x = b[0] + dsp[k][0], y = b[1] + dsp[k][1], z = b[2] + dsp[k][2];
          pbc(s, x, y, z);
          b[0] = x;
          b[1] = y;
          b[2] = z;
        }
      }
      __syncthreads();
    }
    if (threadIdx.x == 0) {
      P.state[r].attempt = att0 + (uint32_t)P.nattempt;
      P.state[r].status = status;
      P.state[r].accepted += nacc;
      P.state[r].attempted += P.nattempt;
      for (int k = 0; k < kMaxSpecies; ++k) P.state[r].epoch[k] = epoch[k];
    }
    __syncthreads();
  }
}

}  // namespace pimc
