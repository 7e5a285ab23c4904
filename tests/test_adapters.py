"""The pi-qmc-side adapters (pi-qmc_gb300/adapters) compile against pi-qmc's
own headers: the integration a maintainer would add is real code, checked
wherever the reference tree exists."""
import os
import subprocess

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = "/root/reference"


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
