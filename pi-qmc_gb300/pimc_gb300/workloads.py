"""Synthetic workloads with the shapes of the benchmark configurations.

No dataset is involved: each workload is a parameter set plus a seeded initial
path.  Parameter names follow pi-qmc's XML attributes / SimulationInfo fields
(species counts, masses, charges, SHO omega, slices, beta, bisection level,
supercell, CoulombAction norder / Ewald cutoffs, node model).

* ``dot2``      2 electrons (1 up, 1 down) in a 3-D harmonic dot, omega=1,
                Coulomb (pair action, norder=3), beta=10, M=256, level 4.
* ``dot20_fn``  20 electrons (10 up, 10 down), SHONodes fixed-node action per
                spin (two 10x10 Slater determinants per slice), beta=20,
                M=1024, level 5.
* ``heg54``     54 electrons (27 up, 27 down) in a cubic box at r_s=4,
                T/T_F=0.5, Ewald Coulomb (|k| < 5 2pi/L), FreeParticleNodes,
                periodic free-particle mover, M=512, level 5.
"""
import math

import numpy as np

DEFAULT_SEED = 20261203
DOT_CELL = 1000.0  # large enough that minimum-image never triggers for a dot


def dot2(**over):
    kw = dict(counts=[1, 1], sho_omega=[1.0, 1.0], nslice=256, beta=10.0, nlevel=4,
              coulomb=1, norder=3, cell=DOT_CELL)
    kw.update(over)
    return kw


def dot20_fn(**over):
    kw = dict(counts=[10, 10], sho_omega=[1.0, 1.0], nslice=1024, beta=20.0, nlevel=5,
              coulomb=1, norder=3, node_kind=[1, 1], node_omega=[1.0, 1.0], cell=DOT_CELL)
    kw.update(over)
    return kw


def heg_box(n, rs):
    return (4.0 * math.pi * n / 3.0) ** (1.0 / 3.0) * rs


def heg54(n=54, nslice=512, nlevel=5, rs=4.0, t_over_tf=0.5, kcut_units=5.0, **over):
    lbox = heg_box(n, rs)
    tf = (9.0 * math.pi / 4.0) ** (2.0 / 3.0) / (2.0 * rs * rs)
    beta = 1.0 / (t_over_tf * tf)
    kw = dict(counts=[n // 2, n - n // 2], nslice=nslice, beta=beta, nlevel=nlevel,
              coulomb=1, norder=3, ewald=1, ewald_kcut=kcut_units * 2.0 * math.pi / lbox,
              cell=lbox, mover=1, node_kind=[2, 2])
    kw.update(over)
    return kw


def initial_path(cfg, kind, seed=DEFAULT_SEED):
    """Initial beads [nslice][npart][3].

    'gauss': every bead N(0,1) per coordinate, independent per slice.
    'const': one N(0,1) point per particle, the same on every slice (a path
             with positive Slater determinants at every slice pair).
    'grid':  constant-in-time paths on a simple-cubic grid filling the box.
    """
    ns, npart = cfg.nslice if hasattr(cfg, "nslice") else cfg["nslice"], None
    npart = cfg.npart if hasattr(cfg, "npart") else sum(cfg["counts"])
    rng = np.random.default_rng(seed)
    if kind == "gauss":
        return rng.normal(size=(ns, npart, 3))
    if kind == "const":
        return np.repeat(rng.normal(size=(1, npart, 3)), ns, axis=0)
    if kind == "grid":
        lbox = cfg.cell[0] if hasattr(cfg, "cell") else cfg["cell"]
        g = int(math.ceil(npart ** (1.0 / 3.0) - 1e-9))
        pts = np.array([[i, j, k] for i in range(g) for j in range(g) for k in range(g)][:npart],
                       float) * (lbox / g) - lbox / 2 + lbox / (2 * g)
        return np.repeat(pts[None], ns, axis=0)
    raise ValueError(kind)


def batch_dots(nrep=4096, seed=DEFAULT_SEED, levels=(4, 5), slices=(128, 256, 512, 1024),
               nmin=2, nmax=32, omega=(0.5, 2.0), tau=1.0 / 25.6):
    """Uneven harmonic-dot replicas: N uniform in {nmin..nmax} (ceil(N/2) up,
    floor(N/2) down, SHONodes on each spin), omega uniform in [0.5, 2], M drawn
    from `slices`, beta = M tau, level drawn from `levels`, Coulomb pair action.
    The node model's temperature attribute is omega/4: at T = 1/beta the
    free-oscillator density matrix is numerically rank-deficient in FP64 once
    omega beta / 2 exceeds ~20 (exp(2 c r_i.r_j) rounds to 1)."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(nrep):
        n = int(rng.integers(nmin, nmax + 1))
        w = float(rng.uniform(*omega))
        m = int(rng.choice(slices))
        lev = int(rng.choice(levels))
        up, dn = (n + 1) // 2, n // 2
        counts = [up, dn] if dn > 0 else [up]
        ns = len(counts)
        out.append(dict(counts=counts, sho_omega=[w] * ns, nslice=m, beta=m * tau, nlevel=lev,
                        coulomb=1, norder=3, node_kind=[1] * ns, node_omega=[w] * ns,
                        node_temperature=w / 4.0, cell=DOT_CELL))
    return out


def tables_for(kw, base_tables):
    """Pair tables of a batch replica taken from one shared table set built for
    a two-species system with both species larger than one (same tau, masses,
    charges and cell): pairs (0,0), (0,1), (1,1) exist as pi-qmc's CoulombAction
    creates them (distinct species, or more than one particle)."""
    counts = kw["counts"]
    by = {tuple(t["species"]): t for t in base_tables}
    out = []
    ns = len(counts)
    for i in range(ns):
        for j in range(i, ns):
            if i != j or counts[i] > 1:
                out.append(by[(i, j)])
    return out


def serve_stream(nreq, rate=200.0, seed=DEFAULT_SEED, sweep_scale=1e-4, nmin=2, nmax=64,
                 slices=(64, 128, 256, 512, 1024, 2048), sweeps=(1e3, 1e5), omega=(0.5, 2.0),
                 tau=1.0 / 25.6):
    """A stream of dot simulations arriving as a Poisson process of `rate`
    requests/s: N uniform in {nmin..nmax} (ceil(N/2) up, floor(N/2) down,
    SHONodes per spin, node temperature omega/4), omega uniform in [0.5, 2],
    M uniform over `slices`, beta = M tau, level 4 for M <= 128 else 5, requested
    sweeps log-uniform in `sweeps` and multiplied by `sweep_scale`.

    Returns [(arrival_seconds, system_kw, sweeps)], sweeps a float >= 0."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for _ in range(nreq):
        t += float(rng.exponential(1.0 / rate))
        n = int(rng.integers(nmin, nmax + 1))
        w = float(rng.uniform(*omega))
        m = int(rng.choice(slices))
        lev = 4 if m <= 128 else 5
        sw = math.exp(rng.uniform(math.log(sweeps[0]), math.log(sweeps[1]))) * sweep_scale
        up, dn = (n + 1) // 2, n // 2
        counts = [up, dn] if dn > 0 else [up]
        ns = len(counts)
        kw = dict(counts=counts, sho_omega=[w] * ns, nslice=m, beta=m * tau, nlevel=lev,
                  coulomb=1, norder=3, node_kind=[1] * ns, node_omega=[w] * ns,
                  node_temperature=w / 4.0, cell=DOT_CELL)
        out.append((t, kw, sw))
    return out


def sweep_attempts(kw):
    """Section attempts of one sweep: every particle's path covered once by
    non-overlapping sections, N M / 2^L attempts."""
    return max(1, sum(kw["counts"]) * kw["nslice"] // (1 << kw["nlevel"]))
