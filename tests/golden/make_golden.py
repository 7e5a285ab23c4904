"""Generate the golden fixtures in tests/golden/ by running pi-qmc's own code.

Runs oracle/_ref/libpimcref.so (pi-qmc's hot-path sources, built from the
reference tree by oracle/build_ref.py) on seeded synthetic inputs and stores:
the configuration, the initial path, the pair-action and Ewald tables the
reference built, per-attempt records (section start, moving particle, rejecting
level, per-level action differences and mover log transition ratios), the
final path (stored as its difference from the initial path, which compresses)
and, on the final path, the thermodynamic, virial (windows 1, 4, 16) and
Coulomb energy estimators (direct, and for periodic cases the optimized-Ewald
estimator together with the Ewald table and short-range grid it built), and
for some cases a recorded run of rigid-displacement moves from the final path
(DisplaceMoveSampler / DoubleDisplaceMoveSampler with a UniformMover).  For two
cases the final path is also written by pi-qmc's WritePaths (<case>.paths) and
read back by its PathReader (path_files.npz).  For the fixed-node cases of
workloads.NODE_CASES, nodes_<case>.npz holds pi-qmc's NodeModel::evaluate and
evaluateDistance (SHONodes, FreeParticleNodes) on seeded slice pairs near the
final path, at the scale the node model reached; for the ill-conditioned SHO dot
(omega/T = 20) it also holds the same determinants and distances evaluated in
60-digit arithmetic (mpmath) from the same double inputs, the exact values the
FP64 implementations are measured against.

The fixtures let machines without the reference tree (the GPU machine) pin the C++
restatement and the CUDA engine against the reference's own outputs.

Usage: python tests/golden/make_golden.py [case ...]   (needs the reference tree;
no case names: every case)
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "oracle"))
sys.path.insert(0, os.path.join(REPO, "tests"))

import oracle_lib as O  # noqa: E402
import workloads as W  # noqa: E402


VIRIAL_WINDOWS = (1, 4, 16)
# rigid-displacement runs from the final path: (box, nmoving, species, attempts)
DISPLACE = {
    "dot2_small": ((0.5, 0.5, 0.5), 1, -1, 60),
    "dot2_full": ((0.6, 0.4, 0.5), 2, -1, 40),
    "dot4_fn": ((0.3, 0.3, 0.3), 2, 1, 40),
    "heg8": ((1.0, 1.0, 1.0), 1, -1, 30),
}



def run_case(name, kw, init, nattempt):
    cfg = O.make_config(**kw)
    ref = O.RefOracle(cfg)
    x0 = W.initial_path(cfg, init)
    ref.set_path(x0)
    tabs = ref.pair_tables()
    ew = ref.ewald_table()
    e0 = ref.thermo_energy()
    recs = ref.run(nattempt)
    x1 = ref.get_path()
    e1 = ref.thermo_energy()
    out = dict(
        config=np.array(repr(kw)), init=np.array(init), nattempt=nattempt,
        path0=x0, dpath=x1 - x0, energy0=e0, energy1=e1,
        npair=len(tabs),
    )
    for k, t in enumerate(tabs):
        s1, s2 = O.species_pair_of(t, cfg)
        out[f"pair{k}_species"] = np.array([s1, s2], np.int32)
        out[f"pair{k}_grid"] = np.array([t["ngpts"], t["norder"]], np.int32)
        out[f"pair{k}_params"] = np.array([t["rgridinv"], t["logrratioinv"]])
        out[f"pair{k}_ugrid"] = t["ugrid"]
    if ew is not None:
        out["ewald_kvec"] = ew["kvec"]
        out["ewald_vk"] = ew["vk"]
        out["ewald_scalars"] = np.array([ew["one_over_2v"], ew["self_energy"]])
        out["ewald_ikmax"] = np.array(ew["ikmax"], np.int32)
        out["ewald_coef"] = ew["coef"]
    for k in ("ifirst1", "ifirst2", "ipart", "reject_level", "ds", "ds_node", "lnt"):
        out["rec_" + k] = recs[k]
    out["naccepted"] = recs["naccepted"]
    out["est_virial_windows"] = np.array(VIRIAL_WINDOWS, np.int32)
    out["est_virial"] = np.array([ref.virial_energy(w) for w in VIRIAL_WINDOWS])
    out["est_coulomb"] = np.array(ref.coulomb_energy(1.0))
    if kw.get("ewald"):
        lbox = kw["cell"] if not isinstance(kw["cell"], (list, tuple)) else kw["cell"][0]
        rcut, kcut = lbox / 2, 5 * 2 * np.pi / lbox
        est, vg = ref.estimator_ewald(1.0, rcut, kcut)
        out["estew_params"] = np.array([1.0, rcut, kcut])
        out["estew_kvec"] = est["kvec"]
        out["estew_vk"] = est["vk"]
        out["estew_scalars"] = np.array([est["one_over_2v"], est["self_energy"]])
        out["estew_ikmax"] = np.array(est["ikmax"], np.int32)
        out["estew_vgrid"] = vg
        out["est_ewald_coulomb"] = np.array(ref.ewald_coulomb_energy(1.0, rcut, kcut))
    if name in DISPLACE:
        box, nmov, species, nd = DISPLACE[name]
        # the chain continues: attempt numbers follow the section attempts
        d = ref.run_displace(nd, box, nmov, species, first_attempt=nattempt)
        out["disp_params"] = np.array([box[0], box[1], box[2], nmov, species, nd, nattempt])
        for k in ("ipart", "disp", "ds", "ds_node", "accepted"):
            out["disp_" + k] = d[k]
        out["disp_dpath"] = ref.get_path() - x1
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **out)
    print(f"{name}: {nattempt} attempts, {recs['naccepted']} accepted, "
          f"E={e1:.6f}, {os.path.getsize(path) / 1024:.0f} KiB")


# restart files: pi-qmc's WritePaths on the final path of these cases, and what
# its PathReader makes of that file and of two variants (no permutation line
# with a wrapped last slice; half the slices, read with bfactor 2)
PATH_FILES = ("dot2_small", "dot4_fn")


def make_path_files():
    out = {}
    for name in PATH_FILES:
        kw, init, n = W.GOLDEN_CASES[name]
        z = np.load(os.path.join(HERE, name + ".npz"))
        x1 = z["path0"] + z["dpath"]
        ref = O.RefOracle(O.make_config(**kw))
        ref.set_path(x1)
        fname = os.path.join(HERE, name + ".paths")
        ref.write_paths(fname)
        lines = open(fname).read().splitlines(keepends=True)
        variants = {name: (fname, 1)}
        if name == "dot4_fn":
            m = kw["nslice"]
            noperm = os.path.join(HERE, name + "_noperm.paths")
            with open(noperm, "w") as f:
                f.writelines(lines[1:] + [lines[2]])
            half = os.path.join(HERE, name + "_half.paths")
            with open(half, "w") as f:
                f.writelines(lines[:2 + m // 2])
            variants[name + "_noperm"] = (noperm, 1)
            variants[name + "_half"] = (half, 2)
        for key, (fn, bfactor) in variants.items():
            ref.set_path(np.zeros_like(x1))
            ref.read_paths(fn, bfactor)
            out[key + "_read"] = ref.get_path()
            out[key + "_bfactor"] = np.array(bfactor)
        out[name + "_path"] = x1
    np.savez_compressed(os.path.join(HERE, "path_files.npz"), **out)
    print("path files:", ", ".join(k[:-5] for k in out if k.endswith("_read")))


NODE_PAIRS = 24
EXACT_DIGITS = 60


def sho_exact(r1, r2, ifirst, n, omega, temperature, mass, tau, scale):
    """SHONodes' determinant and nodal distances (src/fixednode/SHONodes.cc:51-170)
    in EXACT_DIGITS-digit arithmetic from the double inputs: the matrix
    scale exp(-c((r_i^2 + r_j^2) cosh - 2 r_i.r_j)), its determinant, and
    d = sqrt(2m / ((|sum_i inv(j,i) scale grad_ij|^2 + 1e-15) tau)) for both sides."""
    import mpmath as mp
    mp.mp.dps = EXACT_DIGITS
    wt = mp.mpf(omega) * mp.mpf(0.5) / mp.mpf(temperature)
    ch, c = mp.cosh(wt), mp.mpf(mass) * mp.mpf(0.5) * mp.mpf(omega) / mp.sinh(wt)
    S = mp.mpf(scale)
    R1 = [[mp.mpf(float(x)) for x in r1[ifirst + j]] for j in range(n)]
    R2 = [[mp.mpf(float(x)) for x in r2[ifirst + i]] for i in range(n)]
    dot = lambda a, b: a[0] * b[0] + a[1] * b[1] + a[2] * b[2]  # noqa: E731
    E = [[mp.exp(-c * ((dot(R2[i], R2[i]) + dot(R1[j], R1[j])) * ch - 2 * dot(R2[i], R1[j])))
          for j in range(n)] for i in range(n)]
    A = mp.matrix([[S * E[i][j] for j in range(n)] for i in range(n)])
    det = mp.det(A)
    X = A ** -1
    k = 2 * mp.mpf(mass) / mp.mpf(tau)

    def dist(g):
        return float(mp.sqrt(k / (g[0] ** 2 + g[1] ** 2 + g[2] ** 2 + mp.mpf(1e-15))))

    d1 = [dist([sum(X[j, i] * S * 2 * c * (R2[i][d] - ch * R1[j][d]) * E[i][j]
                    for i in range(n)) for d in range(3)]) for j in range(n)]
    d2 = [dist([sum(X[j, i] * S * 2 * c * (R1[j][d] - ch * R2[i][d]) * E[i][j]
                    for j in range(n)) for d in range(3)]) for i in range(n)]
    return float(det), np.array(d1), np.array(d2)


def make_node_fixture(name):
    """pi-qmc's node models on NODE_PAIRS seeded slice pairs (slice t and t + M/2 of
    the final golden path, each coordinate moved by N(0, 0.05^2)), every node
    species, islice 0, at the scale pi-qmc's own set-up rescaling reached."""
    kw, init, n = W.GOLDEN_CASES[name]
    cfg = O.make_config(**kw)
    ref = O.RefOracle(cfg)
    ref.set_path(W.initial_path(cfg, init))
    ref.run(n)
    x1 = ref.get_path()
    M, npart = cfg.nslice, cfg.npart
    rng = np.random.default_rng(4242)
    ts = rng.integers(0, M // 2, NODE_PAIRS)
    r1 = x1[ts] + 0.05 * rng.normal(size=(NODE_PAIRS, npart, 3))
    r2 = x1[ts + M // 2] + 0.05 * rng.normal(size=(NODE_PAIRS, npart, 3))
    out = dict(config=np.array(repr(kw)), r1=r1, r2=r2)
    firsts = np.cumsum([0] + [cfg.spec_count[i] for i in range(cfg.nspecies)])
    for sp in range(cfg.nspecies):
        if not cfg.node_kind[sp]:
            continue
        res = [ref.node_eval(sp, r1[b], r2[b], 0, False) for b in range(NODE_PAIRS)]
        out[f"sp{sp}_scale"] = np.array(ref.node_scale(sp))
        out[f"sp{sp}_err"] = np.array([r[0] for r in res], np.int32)
        out[f"sp{sp}_det"] = np.array([r[1] for r in res])
        out[f"sp{sp}_d1"] = np.array([r[2] for r in res])
        out[f"sp{sp}_d2"] = np.array([r[3] for r in res])
        if name == "dot20_fn":
            ex = [sho_exact(r1[b], r2[b], firsts[sp], cfg.spec_count[sp], cfg.node_omega[sp],
                            cfg.node_temperature, cfg.spec_mass[sp], cfg.tau,
                            ref.node_scale(sp)) for b in range(NODE_PAIRS)]
            out[f"sp{sp}_exact_det"] = np.array([e[0] for e in ex])
            out[f"sp{sp}_exact_d1"] = np.array([e[1] for e in ex])
            out[f"sp{sp}_exact_d2"] = np.array([e[2] for e in ex])
            out[f"sp{sp}_first"] = np.array(firsts[sp])
    path = os.path.join(HERE, "nodes_" + name + ".npz")
    np.savez_compressed(path, **out)
    print(f"nodes_{name}: {NODE_PAIRS} slice pairs, {os.path.getsize(path) / 1024:.0f} KiB")


def make_table_fixture():
    """tables_dot_mix.npz: the pair tables pi-qmc's CoulombAction builds for the
    harmonic-dot mixes (batched replicas, serving stream): tau = 1/25.6, unit
    masses and charges, two species of more than one particle each (pairs
    (0,0), (0,1), (1,1)), the dot cell.  Every replica of those mixes shares
    these tables (their tau, masses and charges are the same)."""
    from pimc_gb300 import workloads as WL
    kw = dict(WL.batch_dots(1)[0], counts=[2, 2], node_kind=[1, 1], node_omega=[1.0, 1.0],
              sho_omega=[1.0, 1.0])
    cfg = O.make_config(**kw)
    ref = O.RefOracle(cfg)
    tabs = ref.pair_tables()
    out = dict(config=np.array(repr(kw)), npair=len(tabs))
    for k, t in enumerate(tabs):
        s1, s2 = O.species_pair_of(t, cfg)
        out[f"pair{k}_species"] = np.array([s1, s2], np.int32)
        out[f"pair{k}_grid"] = np.array([t["ngpts"], t["norder"]], np.int32)
        out[f"pair{k}_params"] = np.array([t["rgridinv"], t["logrratioinv"]])
        out[f"pair{k}_ugrid"] = t["ugrid"]
    path = os.path.join(HERE, "tables_dot_mix.npz")
    np.savez_compressed(path, **out)
    print(f"tables_dot_mix: {len(tabs)} pair tables, {os.path.getsize(path) / 1024:.0f} KiB")


def main(names=()):
    for name, (kw, init, n) in W.GOLDEN_CASES.items():
        if not names or name in names:
            run_case(name, kw, init, n)
    for name in W.NODE_CASES:
        if not names or name in names or ("nodes_" + name) in names:
            make_node_fixture(name)
    if not names or "path_files" in names:
        make_path_files()
    if not names or "tables" in names:
        make_table_fixture()


if __name__ == "__main__":
    main(tuple(sys.argv[1:]))
