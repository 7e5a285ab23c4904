"""Equilibrated thermodynamic energies of pi-qmc's own code, the target the
engine's energies are held to (tests/golden/energy_<case>.npz).

For each case, PROCS independent chains of oracle/_ref (pi-qmc's hot-path
sources built from the reference tree) run in separate processes, each from
its own seeded initial path and random stream: `equil` sweeps are discarded,
then `nblock` blocks of `block` sweeps follow, the ThermoEnergyEstimator value
(src/estimator/ThermoEnergyEstimator.cc:32-66) measured after every sweep (one
sweep = ceil(M / 2^L) * N section attempts, pi-qmc's usual interval).  Every
sweep is followed by DISP rigid displacement attempts of one particle's whole
path (DisplaceMoveSampler / DoubleDisplaceMoveSampler with a UniformMover of
box DISP_BOX): bisection sections move a path's centroid only slowly, and
without them the potential energy decorrelates over many thousands of sweeps
(blocks of 1500 sweeps then understate the error).  The file holds every block
mean; E is their mean and sigma their standard error (PROCS * nblock >= 50
blocks).

Usage: python tests/golden/make_energy.py [case ...]   (needs the reference tree)
"""
import multiprocessing as mp
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "oracle"))
sys.path.insert(0, os.path.join(REPO, "tests"))

PROCS = 8
# case: (golden case whose configuration is used, initial path kind, equil, nblock, block)
CASES = {
    "dot2_full": ("dot2_full", "gauss", 2000, 16, 1500),
    "dot4_fn": ("dot4_fn", "const", 1000, 16, 500),
}
SEED = 5150
DISP, DISP_BOX = 2, 1.0


def sweep_attempts(kw):
    return -(-kw["nslice"] // (1 << kw["nlevel"])) * sum(kw["counts"])


def chain(args):
    name, p = args
    devnull = os.open(os.devnull, os.O_WRONLY)
    os.dup2(devnull, 1)  # pi-qmc's constructors print progress
    import oracle_lib as O
    import workloads as W
    golden, init, equil, nblock, block = CASES[name]
    kw = W.GOLDEN_CASES[golden][0]
    cfg = O.make_config(**dict(kw, seed=SEED, replica=p))
    ref = O.RefOracle(cfg)
    ref.set_path(W.initial_path(cfg, init, seed=SEED + 17 * p))
    sw = sweep_attempts(kw)
    n = 0

    def sweep():
        nonlocal n
        ref.run(sw, first_attempt=n)
        n += sw
        ref.run_displace(DISP, [DISP_BOX] * 3, 1, -1, first_attempt=n)
        n += DISP

    for _ in range(equil):
        sweep()
    means = []
    for _ in range(nblock):
        e = 0.0
        for _ in range(block):
            sweep()
            e += ref.thermo_energy()
        means.append(e / block)
    return means


def make(name):
    golden, init, equil, nblock, block = CASES[name]
    with mp.get_context("spawn").Pool(PROCS) as pool:
        means = np.array(pool.map(chain, [(name, p) for p in range(PROCS)]))
    flat = means.ravel()
    e, sig = float(flat.mean()), float(flat.std(ddof=1) / np.sqrt(flat.size))
    np.savez_compressed(os.path.join(HERE, "energy_" + name + ".npz"), block_means=means,
                        energy=e, sigma=sig, equil=equil, block=block, golden=golden,
                        seed=SEED, init=init, disp=DISP, disp_box=DISP_BOX)
    half = means[:, :nblock // 2].mean() - means[:, nblock // 2:].mean()
    print(f"energy_{name}: E = {e:.6f} +- {sig:.6f} ({flat.size} blocks of {block} sweeps "
          f"after {equil}); first half - second half = {half:+.5f}")


if __name__ == "__main__":
    for name in (sys.argv[1:] or CASES):
        make(name)
