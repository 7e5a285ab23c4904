"""The pi-qmc-side adapters (pi-qmc_gb300/adapters) compile against pi-qmc's
own headers: the integration a maintainer would add is real code, checked
wherever the reference tree exists."""
import os
import subprocess

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("PIMC_REFERENCE_TREE", "/root/reference")


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "src")),
                    reason="pi-qmc source tree not present")
def test_adapters_compile_against_pi_qmc_headers(tmp_path):
    src = os.path.join(REPO, "pi-qmc_gb300", "adapters", "GpuAdapters.cc")
    cmd = ["g++", "-std=gnu++11", "-fsyntax-only", "-w", "-DHAVE_CONFIG_H",
           "-I" + os.path.join(REPO, "oracle", "shim"), "-I" + os.path.join(REF, "src"),
           "-I" + os.path.join(REF, "contrib", "blitz-0.9"),
           "-I" + os.path.join(REPO, "include"), src]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr[-3000:]


@pytest.mark.skipif(not (os.path.isdir(os.path.join(REF, "src")) and
                         os.path.exists(os.path.join(REPO, "oracle", "_ref", "libpimcref.so"))),
                    reason="pi-qmc source tree and its compiled objects not present")
def test_system_from_simulation(tmp_path):
    """systemFromSimulation maps pi-qmc's SimulationInfo and the parser
    attributes onto the engine's system description (linked against pi-qmc's
    own SimulationInfo / Species / SuperCell objects; no GPU call)."""
    import pimc_gb300
    lib = pimc_gb300.build.build()
    refdir = os.path.join(REPO, "oracle", "_ref")
    exe = str(tmp_path / "sys")
    cmd = ["g++", "-std=gnu++11", "-w", "-DHAVE_CONFIG_H",
           "-I" + os.path.join(REPO, "oracle", "shim"), "-I" + os.path.join(REF, "src"),
           "-I" + os.path.join(REF, "contrib", "blitz-0.9"),
           "-I" + os.path.join(REPO, "include"),
           "-I" + os.path.join(REPO, "pi-qmc_gb300", "adapters"),
           os.path.join(REPO, "tests", "adapters", "system_from_simulation.cc"),
           os.path.join(REPO, "pi-qmc_gb300", "adapters", "GpuAdapters.cc"), "-o", exe,
           "-L" + refdir, "-lpimcref", "-Wl,-rpath," + refdir,
           "-L" + os.path.dirname(lib), "-l:" + os.path.basename(lib),
           "-Wl,-rpath," + os.path.dirname(lib)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr[-3000:]
    out = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert out.returncode == 0, out.stderr
    first, second = out.stdout.split("\n")[:2]
    v = first.split()
    # npart nspecies counts masses charges sho_omega node_kind node_omega nslice tau
    # nlevel cell spring coulomb ewald mover
    assert v == ["5", "2", "2", "3", "1", "2", "-1", "1", "1", "2", "1", "2", "1.5", "0", "40",
                 "0.05", "3", "10", "11", "12", "1", "1", "0", "1"]
    assert second == "0.5"  # node temperature: the simulation's
