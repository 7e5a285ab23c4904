"""Build recipe for oracle/_ref/libpimcref.so: pi-qmc's own hot-path sources,
compiled unmodified from the reference tree plus the replay shim (oracle/shim)
and the driver (oracle/ref_driver.cc).  Test infrastructure only.

The reference tree is read where it lies; nothing from it is copied into this
repository, and the output goes only to oracle/_ref/ (git-ignored).  LAPACK
(dgetrf/dgetri/dgetrs/dgesv) comes from scipy's bundled OpenBLAS, whose symbols
carry a ``scipy_`` prefix (see oracle/shim/config.h).

Usage: python oracle/build_ref.py [REFERENCE_ROOT]
(default: $PIMC_REFERENCE_TREE, else /root/reference)
"""
import concurrent.futures as cf
import glob
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")

# The translation units on the bisection / fixed-node / estimator path.
SOURCES = [
    "action/SpringAction.cc", "action/SHOAction.cc", "action/PrimSHOAction.cc",
    "action/CoulombAction.cc", "action/PairAction.cc", "action/ImagePairAction.cc",
    "action/EwaldImagePairAction.cc", "action/CompositeAction.cc",
    "action/CompositeDoubleAction.cc", "action/coulomb/Coulomb1DLinkAction.cpp",
    "action/coulomb/Coulomb3DLinkAction.cpp", "action/coulomb/CoulombLinkAction.cpp",
    "fixednode/FixedNodeAction.cc", "fixednode/SHONodes.cc",
    "fixednode/FreeParticleNodes.cc", "fixednode/NodeModel.cc", "util/Hungarian.cc",
    "util/PeriodicGaussian.cc", "util/SuperCell.cc", "util/EwaldSum.cc",
    "util/OptEwaldSum.cc", "util/TradEwaldSum.cc", "util/Permutation.cc",
    "base/SimulationInfo.cc", "base/Species.cc", "base/BeadFactory.cc",
    "base/SerialPaths.cc", "base/Paths.cc", "advancer/MultiLevelSampler.cc",
    "advancer/DoubleMLSampler.cc", "advancer/SectionChooser.cc",
    "advancer/DoubleSectionChooser.cc", "advancer/mover/FreeMover.cc",
    "advancer/mover/FreeMoverPBC.cc", "advancer/SimpleParticleChooser.cc",
    "advancer/SpeciesParticleChooser.cc", "advancer/ParticleChooser.cc",
    "advancer/PermutationChooser.cc", "stats/AccRejEstimator.cc",
    "estimator/VirialEnergyEstimator.cc", "estimator/CoulombEnergyEstimator.cc",
    "estimator/EwaldCoulombEstimator.cc", "stats/ScalarEstimator.cc",
    "stats/SimpleScalarAccumulator.cpp", "advancer/DisplaceMoveSampler.cc",
    "advancer/DoubleDisplaceMoveSampler.cc", "advancer/UniformMover.cc",
    "algorithm/WritePaths.cc", "algorithm/PathReader.cc",
]

# where the reference tree lies (read-only); the environment variable overrides
DEFAULT_TREE = os.environ.get("PIMC_REFERENCE_TREE", "/root/reference")

FLAGS = ["-std=gnu++98", "-O2", "-fPIC", "-w", "-ffp-contract=off", "-DHAVE_CONFIG_H"]


def openblas():
    import scipy
    libs = glob.glob(os.path.join(os.path.dirname(scipy.__file__), "..", "scipy.libs",
                                  "libscipy_openblas*.so"))
    if not libs:
        raise RuntimeError("scipy-bundled OpenBLAS not found")
    return os.path.abspath(libs[0])


def build(ref_root=DEFAULT_TREE, verbose=False):
    src = os.path.join(ref_root, "src")
    if not os.path.isdir(src):
        raise FileNotFoundError(f"reference tree not found at {ref_root}")
    os.makedirs(OUT, exist_ok=True)
    inc = ["-I" + os.path.join(HERE, "shim"), "-I" + src,
           "-I" + os.path.join(ref_root, "contrib", "blitz-0.9")]
    jobs = []
    for rel in SOURCES:
        obj = os.path.join(OUT, rel.replace("/", "_") + ".o")
        jobs.append(["g++", *FLAGS, *inc, "-c", os.path.join(src, rel), "-o", obj])
    drv_obj = os.path.join(OUT, "ref_driver.o")
    jobs.append(["g++", *FLAGS, "-std=gnu++11", *inc, "-I" + HERE, "-c",
                 os.path.join(HERE, "ref_driver.cc"), "-o", drv_obj])
    with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        for cmd, res in zip(jobs, ex.map(
                lambda c: subprocess.run(c, capture_output=True, text=True), jobs)):
            if res.returncode != 0:
                raise RuntimeError("compile failed: " + " ".join(cmd) + "\n" + res.stderr)
    objs = [j[-1] for j in jobs]
    blas = openblas()
    lib = os.path.join(OUT, "libpimcref.so")
    cmd = ["g++", "-shared", "-o", lib, *objs, blas,
           "-Wl,-rpath," + os.path.dirname(blas)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("link failed:\n" + res.stderr)
    if verbose:
        print("built", lib)
    return lib


if __name__ == "__main__":
    build(sys.argv[1] if len(sys.argv) > 1 else DEFAULT_TREE, verbose=True)
