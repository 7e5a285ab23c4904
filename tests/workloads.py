"""Test-side access to the synthetic workloads, plus the golden-fixture cases."""
import os
import sys

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(REPO, "pi-qmc_gb300"))

from pimc_gb300.workloads import dot2, dot20_fn, heg54, initial_path  # noqa: E402,F401

# name -> (config keywords, initial path kind, attempts)
GOLDEN_CASES = {
    "dot2_small": (dot2(nslice=64), "gauss", 600),
    "dot2_full": (dot2(), "gauss", 400),
    "dot4_fn": (dot20_fn(counts=[2, 2], nslice=64, beta=4.0, nlevel=3), "const", 400),
    "dot20_fn": (dot20_fn(), "const", 40),
    "heg8": (heg54(n=8, nslice=128, nlevel=3), "grid", 150),
    "heg54": (heg54(), "grid", 12),
    # a warmer, coarser electron gas (16 electrons, T/T_F = 1, M = 32): nodal
    # distances of a few tau-lengths, so the free-particle nodal action is
    # nonzero on most attempts and moves cross the nodes now and then
    "heg16_hot": (heg54(n=16, nslice=32, nlevel=3, t_over_tf=1.0), "grid", 800),
    # primitive confinement a r^2 + b r^4 (PrimSHOAction) with a Coulomb pair
    # action, no harmonic action, on three electrons of two species
    "dot3_prim": (dot2(counts=[2, 1], sho_omega=[0.0, 0.0], prim_a=[0.5, 0.3],
                       prim_b=[0.05, 0.1], nslice=64, nlevel=3, beta=4.0), "gauss", 500),
    # pi-qmc's SHO system test (test/system/sho/pimc.xml): one electron,
    # SHOAction omega = 0.5, kT = 1, M = 32, level 5 (a section spans the ring)
    "sho_system": (dot2(counts=[1], sho_omega=[0.5], nslice=32, beta=1.0, nlevel=5, coulomb=0,
                        cell=20.0), "gauss", 600),
    # delayed rejection (<Sample delayedRejection="true">): MultiLevelSampler on
    # the plain dot with defaultSigmaFactor 1.3 and newSigmaFactor 0.6, and
    # DoubleMLSampler on the small fixed-node dot with pi-qmc's defaults (1, 0.75)
    "dot2_dr": (dot2(nslice=64, delayed_rejection=1, sigma_factor=1.3, dr_sigma_factor=0.6),
                "gauss", 600),
    "dot4_dr": (dot20_fn(counts=[2, 2], nslice=64, beta=4.0, nlevel=3, delayed_rejection=1),
                "const", 400),
}

# NodeModel fixtures (tests/golden/nodes_<case>.npz): pi-qmc's own
# NodeModel::evaluate + evaluateDistance on seeded slice pairs near the final
# golden path of these cases
NODE_CASES = ("dot4_fn", "dot20_fn", "heg8", "heg54", "heg16_hot")
