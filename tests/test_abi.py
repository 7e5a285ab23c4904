"""The C-ABI library builds, loads without a GPU, and exports every function
include/pimc_gb300.h declares (no compute calls: this runs anywhere)."""
import ctypes as C
import os
import re

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(REPO, "include", "pimc_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
    names = re.findall(r"^[A-Za-z_][\w \t\*]*?\b(pimc_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    import pimc_gb300
    return C.CDLL(pimc_gb300.build.build())


def test_header_declares_the_entry_points():
    names = declared_functions()
    for must in ("pimc_engine_create", "pimc_run_sections", "pimc_thermo_energy",
                 "pimc_server_admit", "pimc_write_paths", "pimc_set_replica_state",
                 "pimc_node_evaluate_noalloc"):
        assert must in names
    assert len(names) >= 40


def test_every_declared_function_is_exported(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_errors_without_an_engine(lib):
    # argument checks run before any CUDA call
    lib.pimc_last_error.restype = C.c_char_p
    assert lib.pimc_run_sections(None, 1, None) == -1
    assert lib.pimc_last_error()
    assert lib.pimc_write_paths(None, 0, b"x") == -1
    assert lib.pimc_paths_write_file(None, None, 1, 1) == -1


# C struct <-> ctypes Structure of the Python binding
STRUCTS = {"pimc_system": "System", "pimc_pair_table": "PairTable",
           "pimc_ewald_table": "EwaldTable", "pimc_move_record": "MoveRecord",
           "pimc_replica_state": "ReplicaState", "pimc_displace_record": "DisplaceRecord",
           "pimc_launch_config": "LaunchConfig", "pimc_server_config": "ServerConfig"}


def test_binding_structs_match_the_header(tmp_path):
    # Every structure the Python binding passes through the ABI has the C
    # header's size and field offsets (compiled with the host C compiler).
    import shutil
    import subprocess
    import pimc_gb300
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    lines = ["#include <stdio.h>", "#include <stddef.h>", f'#include "{HEADER}"',
             "int main(void) {"]
    for cname, pyname in STRUCTS.items():
        cls = getattr(pimc_gb300, pyname)
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in cls._fields_:
            lines.append(f'  printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-std=c99", str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    got = {}
    for line in out:
        if line:
            a, b, v = line.split()
            got[(a, b)] = int(v)
    for cname, pyname in STRUCTS.items():
        cls = getattr(pimc_gb300, pyname)
        assert got[(cname, "size")] == C.sizeof(cls), cname
        for fname, _ in cls._fields_:
            assert got[(cname, fname)] == getattr(cls, fname).offset, (cname, fname)

