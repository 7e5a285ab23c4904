"""Thermodynamic energies of equilibrated chains against the reference.

* pi-qmc's SHO system test (test/system/sho/test_sho.py:25-32): one electron
  with SHOAction omega = 0.5, kT = 1, M = 32, level 5.  The harmonic link action
  is exact, so the estimator's mean is 3/2 omega coth(omega / 2kT) =
  0.75 coth(0.25) at any M; pi-qmc accepts +-0.08 around it.  The cell is 200
  bohr, not the input's 20: FreeMover takes every new bead to its minimum image,
  so in a 20-bohr cell a bead that strays past 10 bohr lands on the far side of
  the box and the estimator's SHO term, which uses the raw positions, spikes
  (with pi-qmc's own algorithm one chain of these 1024 then averages -667 and
  the mean comes out 2.40 +- 0.66, the engine's value to every digit); the
  analytic value is that of the unbounded oscillator.
* pi-qmc's own equilibrated energies (tests/golden/energy_<case>.npz, made by
  tests/golden/make_energy.py with oracle/_ref) for the plain Coulomb dot of
  config 1 (N=2, beta=10, M=256, L=4) and a small fixed-node dot (N=4,
  SHONodes), each in the FP64 form and in the mixed form.  The criterion is
  |E_engine - E_pi-qmc| <= 2 sqrt(sigma_engine^2 + sigma_pi-qmc^2).

Engine standard errors come from the spread of per-replica means over 512
(1024 for the SHO test) independent replicas, each its own Markov chain,
measured once per sweep after an equilibration, each sweep followed by the
reference run's rigid displacement attempts.
"""
import math

import numpy as np
import pytest

import golden_io
import workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pimc():
    import pimc_gb300
    pimc_gb300.build.build()
    return pimc_gb300


def sweep_attempts(kw):
    return -(-kw["nslice"] // (1 << kw["nlevel"])) * sum(kw["counts"])


def equilibrated_energy(pimc, kw, tables, kind, precision, nrep, equil, measure, attempts,
                        disp=0):
    """Per-replica means over `measure` measurements after `equil` untimed
    steps; a step is `attempts` section attempts and, with `disp`, that many
    rigid displacement attempts of one particle's whole path in a 1-bohr box
    (the protocol of tests/golden/make_energy.py)."""
    class _C:
        nslice, npart, cell = kw["nslice"], sum(kw["counts"]), [kw["cell"]] * 3

    e = pimc.Engine(kw, nrep, tables, None, seed=808, precision=precision)
    e.upload_paths([W.initial_path(_C, kind, seed=3000 + r) for r in range(nrep)])
    if disp:
        for _ in range(equil):
            e.run_sections(attempts)
            e.run_displace(disp, [1.0, 1.0, 1.0], 1, -1)
        E = np.empty((measure, nrep))
        for k in range(measure):
            e.run_sections(attempts)
            e.run_displace(disp, [1.0, 1.0, 1.0], 1, -1)
            E[k] = e.thermo_energy()
    else:
        e.run_steps(attempts, equil, energies=False)
        E = e.run_steps(attempts, measure)  # [measure][nrep]
    acc, att, st = e.replica_status()
    e.close()
    assert np.all(st == 0) and np.all(np.isfinite(E))
    per_rep = E.mean(axis=0)
    return float(per_rep.mean()), float(per_rep.std(ddof=1) / math.sqrt(nrep))


@pytest.mark.parametrize("precision", [0, 1])
def test_sho_system_energy(pimc, precision):
    # pi-qmc's input: 100 thermalising attempts, then a measurement after every
    # attempt (one attempt is one sweep of this one-particle ring).
    g = golden_io.load("sho_system")
    kw = dict(g["kw"], cell=200.0)
    e, sig = equilibrated_energy(pimc, kw, [], "gauss", precision, 1024, 100, 500, 1)
    exact = 0.75 / math.tanh(0.25)
    assert abs(e - exact) <= 0.08, (e, sig)
    assert abs(e - exact) <= 3 * sig, (e, sig, exact)
    assert sig < 0.041  # pi-qmc's own run reaches an error bar of 0.041


@pytest.mark.parametrize("case,kind,equil,measure",
                         [("dot2_full", "gauss", 500, 600), ("dot4_fn", "const", 300, 400)])
@pytest.mark.parametrize("precision", [0, 1])
def test_energy_matches_pi_qmc(pimc, case, kind, equil, measure, precision):
    ref = np.load(golden_io.GOLDEN + "/energy_" + case + ".npz")
    g = golden_io.load(case)
    e, sig = equilibrated_energy(pimc, g["kw"], g["tables"], kind, precision, 512, equil,
                                 measure, sweep_attempts(g["kw"]), disp=int(ref["disp"]))
    er, sr = float(ref["energy"]), float(ref["sigma"])
    assert ref["block_means"].size >= 50
    assert abs(e - er) <= 2 * math.hypot(sig, sr), (case, precision, e, sig, er, sr)
    assert sig <= 0.01 * abs(er)


@pytest.mark.parametrize("precision", [0, 1])
def test_delayed_rejection_energy(pimc, precision):
    # Delayed rejection changes the proposals, not the target: config 1's dot
    # with pi-qmc's delayedRejection (default factors: 1 and newSigmaFactor
    # 0.75) reproduces pi-qmc's equilibrated energy of the same system without
    # it (tests/golden/energy_dot2_full.npz), same protocol, within 2 sigma.
    ref = np.load(golden_io.GOLDEN + "/energy_dot2_full.npz")
    g = golden_io.load("dot2_full")
    kw = dict(g["kw"], delayed_rejection=1)
    e, sig = equilibrated_energy(pimc, kw, g["tables"], "gauss", precision, 512, 500, 600,
                                 sweep_attempts(kw), disp=int(ref["disp"]))
    er, sr = float(ref["energy"]), float(ref["sigma"])
    assert abs(e - er) <= 2 * math.hypot(sig, sr), (precision, e, sig, er, sr)

