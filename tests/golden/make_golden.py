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
read back by its PathReader (path_files.npz).

The fixtures let machines without the reference tree (the GPU machine) pin the C++
restatement and the CUDA engine against the reference's own outputs.

Usage: python tests/golden/make_golden.py   (needs the reference tree)
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


def main():
    for name, (kw, init, n) in W.GOLDEN_CASES.items():
        run_case(name, kw, init, n)
    make_path_files()


if __name__ == "__main__":
    main()
