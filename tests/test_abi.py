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
