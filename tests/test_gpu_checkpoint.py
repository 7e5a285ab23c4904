"""Checkpoints on the GPU: restart files of one replica and the state that
decides its future moves.

* a replica whose exact path and state (random-stream position, counts, node
  scales) move to a fresh engine of the same system and seed continues the
  identical chain: same records and paths, bit for bit;
* pimc_write_paths writes what pimc_paths_write_file makes of the downloaded
  path (the format pinned to pi-qmc's WritePaths by tests/test_path_files.py);
* pimc_read_paths replaces one replica's path with what pimc_paths_read_file
  parses, rebuilds that replica's cached Slater results, and leaves the other
  replicas alone;
* a server slot checkpoints the same way (paths are admitted, not read).
"""
import numpy as np
import pytest

import golden_io

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pimc():
    import pimc_gb300
    pimc_gb300.build.build()
    return pimc_gb300


def engine_for(pimc, g, nreplica, seed=4242):
    return pimc.Engine(g["kw"], nreplica, g["tables"], g["ewald"], seed=seed)


def start_paths(g, nreplica):
    rng = np.random.default_rng(9)
    return [g["path1"] + 0.01 * r * rng.normal(size=g["path1"].shape) if r else g["path1"]
            for r in range(nreplica)]


@pytest.mark.parametrize("case", ["dot2_small", "dot4_fn", "heg8"])
def test_exact_resume(pimc, case):
    g = golden_io.load(case)
    R, k1, k2 = 3, 60, 90
    a = engine_for(pimc, g, R)
    a.upload_paths(start_paths(g, R))
    a.run_sections(k1)
    ra = a.run_sections(k2, records=True)

    b = engine_for(pimc, g, R)
    b.upload_paths(start_paths(g, R))
    b.run_sections(k1)
    paths = b.download_paths()
    states = [b.replica_state(r) for r in range(R)]
    assert all(s["attempt"] == k1 for s in states)

    c = engine_for(pimc, g, R)
    c.upload_paths(paths)
    for r in range(R):
        c.set_replica_state(r, states[r])
    assert [c.replica_state(r) for r in range(R)] == states
    rc = c.run_sections(k2, records=True)
    for key in ("ifirst1", "ifirst2", "ipart", "reject_level", "ds", "ds_node", "lnt"):
        assert np.array_equal(ra[key], rc[key]), key
    for pa, pc in zip(a.download_paths(), c.download_paths()):
        assert np.array_equal(pa, pc)
    assert all(np.array_equal(x, y) for x, y in zip(a.replica_status(), c.replica_status()))


def test_state_of_a_fresh_engine_resumes_nothing(pimc):
    # Setting a replica back to attempt 0 replays its chain from the start.
    g = golden_io.load("dot4_fn")
    e = engine_for(pimc, g, 2)
    e.upload_paths(start_paths(g, 2))
    s0 = e.replica_state(1)
    r1 = e.run_sections(40, records=True)
    e.upload_paths(start_paths(g, 2))
    e.set_replica_state(0, s0)
    e.set_replica_state(1, s0)
    r2 = e.run_sections(40, records=True)
    for key in ("ipart", "reject_level", "ds", "ds_node"):
        assert np.array_equal(r1[key], r2[key]), key


@pytest.mark.parametrize("case", ["heg8", "dot4_fn"])
def test_sections_after_displacement(pimc, case):
    # Displacement moves change every slice; the caches rebuilt after them
    # (structure factors, Slater results) equal those of a freshly uploaded path.
    g = golden_io.load(case)
    R = 2
    a = engine_for(pimc, g, R)
    a.upload_paths(start_paths(g, R))
    a.run_sections(20)
    a.run_displace(25, box=[0.4, 0.4, 0.4])
    paths = a.download_paths()
    states = [a.replica_state(r) for r in range(R)]
    b = engine_for(pimc, g, R)
    b.upload_paths(paths)
    for r in range(R):
        b.set_replica_state(r, states[r])
    ra, rb = a.run_sections(80, records=True), b.run_sections(80, records=True)
    for key in ("ipart", "reject_level", "ds", "ds_node"):
        assert np.array_equal(ra[key], rb[key]), key


def test_write_and_read_paths(pimc, tmp_path):
    g = golden_io.load("dot4_fn")
    R = 3
    e = engine_for(pimc, g, R)
    e.upload_paths(start_paths(g, R))
    e.run_sections(50)
    now = e.download_paths()
    f = tmp_path / "replica1.paths"
    e.write_paths(1, f)
    pimc.write_paths_file(tmp_path / "host.paths", now[1])
    assert f.read_bytes() == (tmp_path / "host.paths").read_bytes()

    # read into replica 0 of a second engine: only that replica changes, and
    # the chain from there equals an engine uploaded with the parsed path
    parsed = pimc.read_paths_file(f, g["path1"].shape[1], g["path1"].shape[0])
    d = engine_for(pimc, g, R, seed=99)
    d.upload_paths(start_paths(g, R))
    d.run_sections(10)
    before = d.download_paths()
    state = [d.replica_state(r) for r in range(R)]
    d.read_paths(0, f)
    after = d.download_paths()
    assert np.array_equal(after[0], parsed)
    assert np.array_equal(after[1], before[1]) and np.array_equal(after[2], before[2])
    ref = engine_for(pimc, g, R, seed=99)
    ref.upload_paths([parsed, before[1], before[2]])
    for r in range(R):
        ref.set_replica_state(r, state[r])
    rd, rr = d.run_sections(60, records=True), ref.run_sections(60, records=True)
    for key in ("ipart", "reject_level", "ds", "ds_node"):
        assert np.array_equal(rd[key], rr[key]), key

    with pytest.raises(pimc.PimcError):
        e.read_paths(R, f)  # no such replica
    with pytest.raises(pimc.PimcError):
        e.read_paths(0, tmp_path / "missing")
    assert np.array_equal(e.download_paths()[0], now[0])


def test_server_slot_checkpoint(pimc, tmp_path):
    from pimc_gb300 import workloads as W
    kw = dict(counts=[2, 2], sho_omega=[1.0, 1.0], nslice=128, beta=5.0, nlevel=4, coulomb=1,
              norder=3, node_kind=[1, 1], node_omega=[1.0, 1.0], node_temperature=0.25,
              cell=W.DOT_CELL)
    tabs, _ = pimc.coulomb_tables(kw)
    p0 = W.initial_path(kw, "const", seed=5)
    srv = pimc.Server(4, 64 << 20, 64, 2048, 5, 32, seed=31)
    slot = srv.admit(kw, tabs, p0, 7, 16)
    for _ in range(3):
        srv.run()
    st = srv.replica_state(slot)
    assert st["attempt"] == 48
    srv.write_paths(slot, tmp_path / "slot.paths")
    pimc.write_paths_file(tmp_path / "host.paths", srv.download_path(slot))
    assert (tmp_path / "slot.paths").read_bytes() == (tmp_path / "host.paths").read_bytes()
    # servers take paths at admission
    assert pimc.lib().pimc_read_paths(srv.h, slot, b"slot.paths", 1) == pimc.PIMC_ERR_INVALID
    # a second server admitting the same path and state continues the chain
    srv2 = pimc.Server(4, 64 << 20, 64, 2048, 5, 32, seed=31)
    slot2 = srv2.admit(kw, tabs, srv.download_path(slot), 7, 16)
    srv2.set_replica_state(slot2, st)
    for _ in range(2):
        srv.run()
        srv2.run()
    assert np.array_equal(srv.download_path(slot), srv2.download_path(slot2))
    with pytest.raises(pimc.PimcError):
        srv.replica_state(3)  # slot not in use
