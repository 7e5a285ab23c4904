"""Restart files (pi-qmc_gb300/csrc/paths_io.cc) against pi-qmc's own WritePaths
(src/algorithm/WritePaths.cc:25-114) and PathReader
(src/algorithm/PathReader.cc:20-140): the files pi-qmc wrote for two golden
paths must come out byte for byte, and every file must read back to the same
doubles PathReader gave.  Host code only; no GPU."""
import os

import numpy as np
import pytest

import golden_io

GOLDEN = golden_io.GOLDEN


@pytest.fixture(scope="module")
def pimc():
    import pimc_gb300
    pimc_gb300.build.build()
    return pimc_gb300


@pytest.fixture(scope="module")
def fixtures():
    return np.load(os.path.join(GOLDEN, "path_files.npz"))


@pytest.mark.parametrize("case", ["dot2_small", "dot4_fn"])
def test_writer_matches_reference_bytes(pimc, fixtures, tmp_path, case):
    out = tmp_path / "p.txt"
    pimc.write_paths_file(out, fixtures[case + "_path"])
    assert out.read_bytes() == open(os.path.join(GOLDEN, case + ".paths"), "rb").read()


@pytest.mark.parametrize("key,fname", [("dot2_small", "dot2_small"), ("dot4_fn", "dot4_fn"),
                                       ("dot4_fn_noperm", "dot4_fn_noperm"),
                                       ("dot4_fn_half", "dot4_fn_half")])
def test_reader_matches_reference(pimc, fixtures, key, fname):
    ref = fixtures[key + "_read"]
    bfactor = int(fixtures[key + "_bfactor"])
    x = pimc.read_paths_file(os.path.join(GOLDEN, fname + ".paths"), ref.shape[1], ref.shape[0],
                             bfactor)
    assert np.array_equal(x.view(np.int64), ref.view(np.int64))


def test_write_read_write_is_idempotent(pimc, tmp_path):
    rng = np.random.default_rng(11)
    x = rng.normal(size=(16, 5, 3)) * np.array([1.0, 1e-9, 3e7])
    x[0, 0, 0], x[1, 1, 1], x[2, 2, 2] = -0.0, 1e-300, 5.0
    a, b = tmp_path / "a", tmp_path / "b"
    pimc.write_paths_file(a, x)
    y = pimc.read_paths_file(a, 5, 16)
    pimc.write_paths_file(b, y)
    assert a.read_bytes() == b.read_bytes()
    # 15 significant digits: the values come back to within half an ulp of that
    assert np.all(np.abs(y - x) <= 5e-15 * np.abs(x))


def _expect_invalid(pimc, path, npart, nslice, bfactor=1):
    x = np.full((nslice, npart, 3), 7.0)
    rc = pimc.lib().pimc_paths_read_file(os.fsencode(str(path)), pimc._dp(x), npart, nslice,
                                         bfactor)
    assert rc == pimc.PIMC_ERR_INVALID
    assert np.all(x == 7.0), "a rejected file leaves the path unchanged"
    assert pimc.lib().pimc_last_error()


def test_reader_rejects_bad_files(pimc, tmp_path):
    good = open(os.path.join(GOLDEN, "dot4_fn.paths")).read().splitlines(keepends=True)
    n, m = 4, 64
    cases = {
        "permuted": ["#Permutations 1 0 2 3 \n"] + good[1:],
        "truncated": good[:-1],
        "no_wrap_slice": good[1:],  # no permutation line and no wrapped slice
        "not_a_number": good[:5] + [good[5].replace(good[5].split()[3], "abc", 1)] + good[6:],
        "nonfinite": good[:5] + [good[5].replace(good[5].split()[3], "nan", 1)] + good[6:],
        "empty": [],
    }
    for name, lines in cases.items():
        p = tmp_path / name
        p.write_text("".join(lines))
        _expect_invalid(pimc, p, n, m)
    _expect_invalid(pimc, tmp_path / "missing", n, m)
    _expect_invalid(pimc, os.path.join(GOLDEN, "dot4_fn.paths"), n, m, bfactor=3)  # 64 % 3


def test_wrapped_permutation_detected(pimc, tmp_path):
    """Without a permutation line PathReader matches the wrapped slice to the
    first one; a swapped pair is a permutation the engine rejects."""
    good = open(os.path.join(GOLDEN, "dot4_fn.paths")).read().splitlines(keepends=True)
    first = good[2].split()
    swapped = first[3:6] + first[0:3] + first[6:]
    p = tmp_path / "swap"
    p.write_text("".join(good[1:] + [" ".join(swapped) + " \n"]))
    _expect_invalid(pimc, p, 4, 64)
    p.write_text("".join(good[1:] + [good[2]]))
    x = pimc.read_paths_file(p, 4, 64)
    assert np.array_equal(x, pimc.read_paths_file(os.path.join(GOLDEN, "dot4_fn.paths"), 4, 64))


@pytest.mark.skipif(not __import__("oracle_lib").RefOracle.available(),
                    reason="needs the reference build (oracle/_ref)")
def test_against_reference_objects(pimc, tmp_path):
    """Random paths with awkward values through the reference objects themselves."""
    import oracle_lib as O
    cfg = O.make_config(counts=[2, 1], nslice=8, nlevel=2, beta=0.8)
    ref = O.RefOracle(cfg)
    rng = np.random.default_rng(5)
    for trial in range(4):
        x = rng.normal(size=(8, 3, 3)) * 10.0 ** rng.integers(-12, 12, size=(8, 3, 3))
        x[trial, 0, 0] = -0.0
        x[trial, 1, 2] = float(trial)
        ref.set_path(x)
        ref.write_paths(tmp_path / "ref")
        pimc.write_paths_file(tmp_path / "ours", x)
        assert (tmp_path / "ref").read_bytes() == (tmp_path / "ours").read_bytes()
        ref.set_path(np.zeros_like(x))
        ref.read_paths(tmp_path / "ref")
        y = pimc.read_paths_file(tmp_path / "ref", 3, 8)
        assert np.array_equal(y.view(np.int64), ref.get_path().reshape(8, 3, 3).view(np.int64))
