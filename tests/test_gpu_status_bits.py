"""Failures injected on the host, through pimc_upload_paths: bad paths become
per-replica status bits (pi-qmc's exit-on-error paths,
src/fixednode/FixedNodeAction.cc:342-349 and src/fixednode/SHONodes.cc:86-111,
print and exit instead), the other replicas of the launch run exactly as they
would without the bad one, and nothing traps: every engine call returns PIMC_OK
and the context stays usable.

Each case uploads three replicas, the middle one bad, and compares replicas 0
and 2 bit for bit with an engine whose middle replica is a good path.
"""
import numpy as np
import pytest

import golden_io
import oracle_lib as O
import workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pimc():
    import pimc_gb300
    pimc_gb300.build.build()
    return pimc_gb300


def run_three(pimc, case, bad_path, nattempt):
    g = golden_io.load(case)
    good = [W.initial_path(O.make_config(**g["kw"]), "const" if case == "dot4_fn" else "gauss",
                           seed=70 + r) for r in range(3)]
    out = []
    for middle in (good[1], bad_path(good[1])):
        e = pimc.Engine(g["kw"], 3, g["tables"], g["ewald"], seed=31)
        e.upload_paths([good[0], middle, good[2]])
        st_upload = e.replica_status()[2].copy()
        rec = e.run_sections(nattempt, records=True)
        acc, att, st = e.replica_status()
        out.append(dict(rec=rec, paths=e.download_paths(), status=st, upload_status=st_upload,
                        energy=e.thermo_energy(), attempted=att))
        e.close()
    return out


def assert_others_unaffected(clean, bad):
    for r in (0, 2):
        for k in ("ifirst1", "ipart", "reject_level", "ds", "ds_node", "lnt"):
            assert np.array_equal(clean["rec"][k][r], bad["rec"][k][r]), (r, k)
        assert np.array_equal(clean["paths"][r], bad["paths"][r])
        assert clean["energy"][r] == bad["energy"][r]
        assert bad["status"][r] == 0


@pytest.mark.parametrize("case", ["dot2_small", "dot4_fn"])
def test_nonfinite_coordinate(pimc, case):
    # A NaN bead is reported at upload (PIMC_STATUS_NONFINITE); the replica's
    # moves still run in bounds.
    def bad(p):
        q = p.copy()
        q[7, 1, 2] = np.nan
        return q
    clean, broken = run_three(pimc, case, bad, 120)
    assert clean["status"][1] == 0
    assert broken["upload_status"][1] & pimc.PIMC_STATUS_NONFINITE
    assert broken["status"][1] & pimc.PIMC_STATUS_NONFINITE
    assert broken["attempted"][1] == 120
    assert_others_unaffected(clean, broken)


def test_crossed_node_initial_path(pimc):
    # Two same-spin electrons exchanged on path slices 16..31 of 64: the slice
    # pairs (t, t + M/2) that hold the exchanged slices on one side only change
    # the sign of the up-spin determinant, so the set-up of any section across
    # slice 16 or 32 meets a node crossing (PIMC_STATUS_INIT_CROSSING), where
    # FixedNodeAction::initialize prints "crossed node" and counts towards exit.
    def bad(p):
        q = p.copy()
        q[16:32, [0, 1]] = p[16:32, [1, 0]]
        return q
    clean, broken = run_three(pimc, "dot4_fn", bad, 200)
    assert clean["status"][1] == 0
    assert broken["upload_status"][1] == 0
    assert broken["status"][1] & pimc.PIMC_STATUS_INIT_CROSSING
    assert_others_unaffected(clean, broken)
