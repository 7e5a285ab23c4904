"""Energies of the mixed-precision form against the FP64 form.

The mixed form (FP32 pair-action and nodal-action terms summed in FP64, FP32
Box-Muller proposals, FP64 determinants) must give the same thermodynamic
energy as the FP64 form within two standard errors.  Both run the same replicas
from the same paths and counter streams (the proposals differ in their FP32
transform, so the chains separate); each standard error comes from the spread
over independent replicas after equilibration.  Tolerance:
|E_mixed - E_fp64| <= 2 sqrt(sigma_mixed^2 + sigma_fp64^2).
"""
import math

import numpy as np
import pytest

import workloads as W

pytestmark = pytest.mark.gpu


def run(pimc, kw, tabs, paths, precision, nrep, steps, attempts):
    e = pimc.Engine(kw, nrep, tabs, None, seed=4242, precision=precision)
    e.upload_paths(paths)
    e.run_steps(attempts, steps // 2, energies=False)  # equilibration
    E = e.run_steps(attempts, steps - steps // 2)    # [steps][replicas]
    e.close()
    per_rep = E.mean(axis=0)
    return per_rep.mean(), per_rep.std(ddof=1) / math.sqrt(nrep), per_rep


@pytest.mark.parametrize("name,kw", [
    ("dot4_fn", W.dot20_fn(counts=[2, 2], nslice=64, beta=4.0, nlevel=3)),
    ("dot2", W.dot2(nslice=128)),
])
def test_mixed_energy_within_two_sigma(name, kw):
    import pimc_gb300 as pimc
    tabs, _ = pimc.coulomb_tables(kw)
    nrep = 512
    kind = "const" if any(kw.get("node_kind", [0])) else "gauss"

    class _C:
        nslice, npart, cell = kw["nslice"], sum(kw["counts"]), [kw["cell"]] * 3

    paths = [W.initial_path(_C, kind, seed=900 + r) for r in range(nrep)]
    sweep = sum(kw["counts"]) * kw["nslice"] // (1 << kw["nlevel"])
    e64, s64, r64 = run(pimc, kw, tabs, paths, pimc.PIMC_PREC_FP64, nrep, 40, sweep)
    emx, smx, rmx = run(pimc, kw, tabs, paths, pimc.PIMC_PREC_MIXED, nrep, 40, sweep)
    assert np.all(np.isfinite(r64)) and np.all(np.isfinite(rmx))
    assert s64 > 0
    assert abs(emx - e64) <= 2 * math.hypot(s64, smx), (name, emx, e64, s64, smx)
