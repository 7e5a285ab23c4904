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
}
