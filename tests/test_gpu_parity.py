"""Parity of the CUDA engine with the CPU checkers, through the C ABI.

Inputs are the golden fixtures made by pi-qmc's own code (tests/golden) and
seeded synthetic sections; the checker is the C++ restatement (oracle/port.cc),
itself pinned to the reference by tests/test_oracle.py.

Tolerances: plain action differences and mover ratios 1e-12 relative (to
max(|value|, 1)); section-move decisions (section start, particle, rejecting
level) exact; paths 1e-12; node-model terms 1e-10 relative, except the
omega/T = 20 SHO dot whose Slater matrices have condition numbers 1e12 - 3e13:
there every FP64 implementation (pi-qmc's, the restatement, this engine) is
held to 2e-3 relative of the 60-digit values and of each other (the study is in
tests/test_oracle.py), with exact decisions.
"""
import numpy as np
import pytest

import golden_io
import oracle_lib as O
import workloads as W

pytestmark = pytest.mark.gpu

NODE_TOL = {"dot20_fn": 2e-3}
EXACT_TOL = 2e-3


def rel_close(a, b, tol, floor=1.0):
    return np.all(np.abs(a - b) <= tol * np.maximum(np.abs(a), floor))


@pytest.fixture(scope="module")
def pimc():
    import pimc_gb300
    pimc_gb300.build.build()
    return pimc_gb300


def engine_for(pimc, g, nreplica=1, seed=20261203):
    return pimc.Engine(g["kw"], nreplica, g["tables"], g["ewald"], seed=seed)


def test_streams_bit_exact(pimc):
    # The engine's uniforms and normals equal the CPU replay bit for bit.
    for rep, att in [(0, 0), (3, 17), (4095, 123456)]:
        u, z = pimc.stream_sample(20261203, rep, att, 256)
        cu, cz = O.cpu_stream(20261203, rep, att, 256)
        assert np.array_equal(u, cu)
        assert np.array_equal(z, cz)


@pytest.mark.parametrize("case", list(W.GOLDEN_CASES))
def test_sampler_matches_golden(pimc, case):
    g = golden_io.load(case)
    e = engine_for(pimc, g)
    e.upload_paths([g["path0"]])
    rec = e.run_sections(g["nattempt"], records=True)
    ref = g["records"]
    for k in ("ifirst1", "ifirst2", "ipart", "reject_level"):
        assert np.array_equal(rec[k][0], ref[k]), k
    nl = g["kw"]["nlevel"] + 1
    assert rel_close(rec["ds"][0][:, :nl], ref["ds"][:, :nl], 1e-12)
    assert rel_close(rec["lnt"][0][:, :nl], ref["lnt"][:, :nl], 1e-12)
    assert rel_close(rec["ds_node"][0][:, :nl], ref["ds_node"][:, :nl],
                     NODE_TOL.get(case, 1e-10))
    path = e.download_paths()[0]
    assert np.abs(path - g["path1"]).max() <= 1e-12
    acc, att, st = e.replica_status()
    assert acc[0] == g["naccepted"] and att[0] == g["nattempt"]
    assert e.thermo_energy()[0] == pytest.approx(g["energy1"], rel=1e-12)


@pytest.mark.parametrize("case", ["dot4_fn", "heg8"])
def test_upload_rebuilds_only_what_changed(pimc, case):
    # pimc_upload_paths rebuilds only the cached results (Slater entries,
    # structure factors) that depend on a changed slice.  Uploading the chain's
    # own paths changes nothing: the chain continues bit for bit as without the
    # upload.  Uploading paths with a few slices moved gives what an engine that
    # rebuilt everything from those paths gives, bit for bit.
    g = golden_io.load(case)
    a, b, c = (engine_for(pimc, g) for _ in range(3))
    for e in (a, b):
        e.upload_paths([g["path0"]])
        e.run_sections(60)
    a.upload_paths(a.download_paths())
    ra, rb = a.run_sections(80, records=True), b.run_sections(80, records=True)
    for k in ("reject_level", "ipart", "ds", "ds_node", "lnt"):
        assert np.array_equal(ra[k], rb[k]), k
    x = a.download_paths()[0].copy()
    rng = np.random.default_rng(11)
    for t in rng.choice(x.shape[0], 5, replace=False):
        x[t] += 0.02 * rng.normal(size=x[t].shape)
    a.upload_paths([x])
    c.set_replica_state(0, a.replica_state(0))
    c.upload_paths([x])  # a new engine: every cached result built from x
    ra, rc = a.run_sections(80, records=True), c.run_sections(80, records=True)
    for k in ("reject_level", "ipart", "ds", "ds_node", "lnt"):
        assert np.array_equal(ra[k], rc[k]), k
    assert np.array_equal(a.download_paths()[0], c.download_paths()[0])


def test_replicas_follow_their_own_streams(pimc):
    # Replica r of an engine reproduces the checker run with replica id r.
    g = golden_io.load("dot2_small")
    R = 5
    e = engine_for(pimc, g, nreplica=R, seed=777)
    paths = [W.initial_path(O.make_config(**g["kw"]), "gauss", seed=100 + r) for r in range(R)]
    e.upload_paths(paths)
    rec = e.run_sections(200, records=True)
    out = e.download_paths()
    for r in range(R):
        cfg = O.make_config(**dict(g["kw"], seed=777, replica=r))
        port = O.PortOracle(cfg, g["tables"], g["ewald"])
        port.set_path(paths[r])
        pr = port.run(200)
        assert np.array_equal(pr["reject_level"], rec["reject_level"][r])
        assert np.array_equal(pr["ipart"], rec["ipart"][r])
        assert rel_close(pr["ds"], rec["ds"][r][:, :9], 1e-12)
        assert np.abs(port.get_path() - out[r]).max() <= 1e-12


def test_second_launch_continues_the_chain(pimc):
    # Two launches of n attempts equal one launch of 2n (attempt counters persist).
    g = golden_io.load("dot2_small")
    a = engine_for(pimc, g)
    b = engine_for(pimc, g)
    a.upload_paths([g["path0"]])
    b.upload_paths([g["path0"]])
    a.run_sections(300)
    a.run_sections(300)
    b.run_sections(600)
    assert np.array_equal(a.download_paths()[0], b.download_paths()[0])


@pytest.mark.parametrize("case", ["dot2_small", "heg8", "dot3_prim"])
def test_action_difference_every_level(pimc, case):
    g = golden_io.load(case)
    cfg = O.make_config(**g["kw"])
    port = O.PortOracle(cfg, g["tables"], g["ewald"])
    e = engine_for(pimc, g)
    rng = np.random.default_rng(3)
    nsec = (1 << cfg.nlevel) + 1
    nb = 24
    secs = g["path0"][:nsec][None].repeat(nb, 0) + 0.05 * rng.normal(size=(nb, nsec, cfg.npart, 3))
    ips = rng.integers(0, cfg.npart, nb)
    movs = np.stack([secs[b, :, ips[b], :] for b in range(nb)])
    movs[:, 1:-1] += 0.2 * rng.normal(size=(nb, nsec - 2, 3))
    for level in range(cfg.nlevel + 1):
        ds = e.action_difference(level, secs, movs, ips)
        for b in range(nb):
            ref = port.action_diff(level, secs[b], movs[b], int(ips[b]))
            assert abs(ds[b] - ref) <= 1e-12 * max(abs(ref), 1.0), (level, b)


@pytest.mark.parametrize("case", ["dot4_fn", "heg8"])
def test_node_evaluate(pimc, case):
    g = golden_io.load(case)
    cfg = O.make_config(**g["kw"])
    port = O.PortOracle(cfg, g["tables"], g["ewald"])
    e = engine_for(pimc, g)
    rng = np.random.default_rng(9)
    nb = 16
    base = g["path0"][0]
    r1 = base[None] + 0.3 * rng.normal(size=(nb, cfg.npart, 3))
    r2 = base[None] + 0.3 * rng.normal(size=(nb, cfg.npart, 3))
    for sp in range(cfg.nspecies):
        err, det, d1, d2 = e.node_evaluate(sp, r1, r2)
        for b in range(nb):
            perr, pdet, pd1, pd2 = port.node_eval(sp, r1[b], r2[b], 0, False)
            assert err[b] == perr
            assert abs(det[b] - pdet) <= 1e-10 * abs(pdet)
            assert rel_close(d1[b], pd1, 1e-10)
            assert rel_close(d2[b], pd2, 1e-10)


@pytest.mark.parametrize("case", list(W.NODE_CASES))
def test_node_models_match_golden(pimc, case):
    # The engine's SHONodes / FreeParticleNodes (pimc_node_evaluate) on pi-qmc's
    # own NodeModel::evaluate + evaluateDistance outputs: same slice pairs, the
    # scale pi-qmc's set-up reached; the ill-conditioned dot also against the
    # 60-digit values of the same inputs.
    z = golden_io.load_nodes(case)
    g = golden_io.load(case)
    cfg = O.make_config(**z["kw"])
    e = engine_for(pimc, g)
    st = e.replica_state(0)
    for sp, ref in z["species"].items():
        st["node_scale"][sp] = ref["scale"]
    e.set_replica_state(0, st)
    tol = NODE_TOL.get(case, 1e-10)
    for sp, ref in z["species"].items():
        err, det, d1, d2 = e.node_evaluate(sp, z["r1"], z["r2"])
        assert np.array_equal(err, ref["err"])
        assert np.all(np.abs(det - ref["det"]) <= tol * np.abs(ref["det"])), sp
        assert rel_close(d1, ref["d1"], tol, floor=0.0), sp
        assert rel_close(d2, ref["d2"], tol, floor=0.0), sp
        if "exact_det" in ref:
            f, n = ref["first"], cfg.spec_count[sp]
            assert np.all(np.abs(det - ref["exact_det"]) <= EXACT_TOL * np.abs(ref["exact_det"]))
            assert rel_close(d1[:, f:f + n], ref["exact_d1"], EXACT_TOL, floor=0.0)
            assert rel_close(d2[:, f:f + n], ref["exact_d2"], EXACT_TOL, floor=0.0)


def test_ill_conditioned_dot_matches_checker(pimc):
    # The headline fixed-node dot (N=20, SHONodes, M=1024, L=5) run by the engine
    # and by the restatement from the same path and streams: decisions exact,
    # plain action differences 1e-12, node terms within the conditioning bar.
    g = golden_io.load("dot20_fn")
    cfg = O.make_config(**g["kw"])
    e = engine_for(pimc, g)
    e.upload_paths([g["path1"]])
    rec = e.run_sections(60, records=True)
    port = O.PortOracle(cfg, g["tables"], g["ewald"])
    port.set_path(g["path1"])
    pr = port.run(60)
    for k in ("ifirst1", "ifirst2", "ipart", "reject_level"):
        assert np.array_equal(rec[k][0], pr[k]), k
    nl = g["kw"]["nlevel"] + 1
    assert rel_close(rec["ds"][0][:, :nl], pr["ds"][:, :nl], 1e-12)
    assert rel_close(rec["ds_node"][0][:, :nl], pr["ds_node"][:, :nl], NODE_TOL["dot20_fn"])
    assert np.abs(e.download_paths()[0] - port.get_path()).max() <= 1e-12


def test_thermo_energy_matches_checker(pimc):
    for case in ("dot2_full", "heg8"):
        g = golden_io.load(case)
        e = engine_for(pimc, g)
        e.upload_paths([g["path1"]])
        assert e.thermo_energy()[0] == pytest.approx(g["energy1"], rel=1e-12)


def test_kernel_launch_count(pimc):
    g = golden_io.load("dot2_small")
    e = engine_for(pimc, g)
    e.upload_paths([g["path0"]])
    n0 = e.kernel_launches
    e.run_sections(10)
    e.run_sections(10)
    assert e.kernel_launches - n0 == 2


@pytest.mark.parametrize("case", ["dot4_fn", "heg8"])
def test_slater_cache_is_exact(pimc, case):
    # Cached Slater results stand in for re-evaluations bit for bit: a chain
    # whose cache is wiped every 25 attempts (uploading the paths invalidates
    # it) equals an uninterrupted chain.
    g = golden_io.load(case)
    a = engine_for(pimc, g)
    b = engine_for(pimc, g)
    a.upload_paths([g["path0"]])
    b.upload_paths([g["path0"]])
    ra = a.run_sections(150, records=True)
    rb = []
    for _ in range(6):
        rb.append(b.run_sections(25, records=True))
        b.upload_paths(b.download_paths())
    for k in ("reject_level", "ipart", "ifirst1"):
        assert np.array_equal(ra[k][0], np.concatenate([r[k][0] for r in rb]))
    assert np.array_equal(ra["ds_node"][0], np.concatenate([r["ds_node"][0] for r in rb]))
    # (heg8: the Ewald term comes from the cached structure factors, which a
    # rebuild reproduces bit for bit)
    assert np.array_equal(ra["ds"][0], np.concatenate([r["ds"][0] for r in rb]))
    assert np.array_equal(a.download_paths()[0], b.download_paths()[0])


def test_uneven_batch_matches_checker(pimc):
    # Replicas of different N, M, L, omega in one launch (the batched form):
    # each replica r reproduces the checker run with stream r.
    from pimc_gb300 import workloads as WL
    kws = WL.batch_dots(nrep=10, seed=7, levels=(3, 4), slices=(64, 128), nmax=9)
    base, _ = pimc.coulomb_tables(dict(kws[0], counts=[2, 2], node_kind=[1, 1],
                                       node_omega=[1.0, 1.0], sho_omega=[1.0, 1.0]))
    tabs = [WL.tables_for(kw, base) for kw in kws]
    eng = pimc.Engine.batch(kws, tabs, seed=99)
    paths = [W.initial_path(O.make_config(**kw), "const", seed=500 + r)
             for r, kw in enumerate(kws)]
    eng.upload_paths(paths)
    n = 120
    rec = eng.run_sections(n, records=True)
    out = eng.download_paths()
    E = eng.thermo_energy()
    for r, kw in enumerate(kws):
        cfg = O.make_config(**dict(kw, seed=99, replica=r))
        port = O.PortOracle(cfg, tabs[r], None)
        port.set_path(paths[r])
        pr = port.run(n)
        assert np.array_equal(pr["reject_level"], rec["reject_level"][r]), r
        assert np.array_equal(pr["ipart"], rec["ipart"][r]), r
        assert rel_close(pr["ds"], rec["ds"][r][:, :9], 1e-12)
        assert rel_close(pr["ds_node"], rec["ds_node"][r][:, :9], 1e-9)
        assert np.abs(port.get_path() - out[r]).max() <= 1e-12
        assert E[r] == pytest.approx(port.thermo_energy(), rel=1e-12)


@pytest.mark.parametrize("precision", [0, 1])
def test_largest_node_species_matches_checker(pimc, precision):
    # 32 particles per spin species, the lane-group limit (W = 32, largest
    # Slater scratch), SHONodes at the serving workload's node temperature.
    from pimc_gb300 import workloads as WL
    kw = dict(counts=[32, 32], sho_omega=[1.0, 1.0], nslice=64, beta=64 / 25.6, nlevel=3,
              coulomb=1, norder=3, node_kind=[1, 1], node_omega=[1.0, 1.0],
              node_temperature=0.25, cell=WL.DOT_CELL)
    tabs, _ = pimc.coulomb_tables(kw)
    path = W.initial_path(O.make_config(**kw), "const", seed=41)
    e = pimc.Engine(kw, 2, tabs, None, seed=5, precision=precision)
    e.upload_paths([path, path])
    n = 40
    rec = e.run_sections(n, records=True)
    out = e.download_paths()
    for r in range(2):
        port = O.PortOracle(O.make_config(**dict(kw, seed=5, replica=r)), tabs, None)
        port.set_path(path)
        pr = port.run(n)
        if precision == 0:
            assert np.array_equal(pr["reject_level"], rec["reject_level"][r])
            assert np.array_equal(pr["ipart"], rec["ipart"][r])
            assert rel_close(pr["ds"], rec["ds"][r][:, :9], 1e-12)
            # 32 x 32 SHO Slater matrices: condition numbers ~1e8, so the node
            # terms agree with the checker's LAPACK-order LU to ~1e-8
            assert rel_close(pr["ds_node"], rec["ds_node"][r][:, :9], 1e-6)
            assert np.abs(port.get_path() - out[r]).max() <= 1e-12
        else:
            # the mixed form draws other proposals: same particles and
            # sections, a valid chain (finite action differences)
            assert np.array_equal(pr["ipart"], rec["ipart"][r])
            assert np.all(np.isfinite(rec["ds"][r][:, :5]))
    acc, att, st = e.replica_status()
    assert np.all(att == n) and np.all(st == 0)


@pytest.mark.parametrize("block", [256, 128])
def test_largest_matrices_at_level_5_match_checker(pimc, block):
    # 32 + 32 particles, level 5 (the serving mix's largest requests): at 8
    # warps the Slater scratch lives in global memory, at 4 warps the LU and
    # inverse fit in shared memory; both reproduce the checker's decisions.
    from pimc_gb300 import workloads as WL
    kw = dict(counts=[32, 32], sho_omega=[1.0, 1.0], nslice=128, beta=128 / 25.6, nlevel=5,
              coulomb=1, norder=3, node_kind=[1, 1], node_omega=[1.0, 1.0],
              node_temperature=0.25, cell=WL.DOT_CELL)
    tabs, _ = pimc.coulomb_tables(kw)
    path = W.initial_path(O.make_config(**kw), "const", seed=43)
    e = pimc.Engine(kw, 1, tabs, None, seed=6)
    e.configure(block, 0, 0, 2)
    e.upload_paths([path])
    n = 30
    rec = e.run_sections(n, records=True)
    port = O.PortOracle(O.make_config(**dict(kw, seed=6, replica=0)), tabs, None)
    port.set_path(path)
    pr = port.run(n)
    assert np.array_equal(pr["reject_level"], rec["reject_level"][0])
    assert np.array_equal(pr["ipart"], rec["ipart"][0])
    assert rel_close(pr["ds"], rec["ds"][0][:, :9], 1e-12)
    assert rel_close(pr["ds_node"], rec["ds_node"][0][:, :9], 1e-6)
    assert np.abs(port.get_path() - e.download_paths()[0]).max() <= 1e-12


def test_graph_steps_equal_direct_calls(pimc):
    # The captured step graph (sweep + energy measurement, replayed) is the same
    # work as the direct calls: energies and paths bit for bit, and a replay
    # continues the chain.
    g = golden_io.load("dot4_fn")
    a = engine_for(pimc, g, nreplica=3)
    b = engine_for(pimc, g, nreplica=3)
    for e in (a, b):
        e.upload_paths([g["path0"]] * 3)
    ea = np.concatenate([a.run_steps(20, 3), a.run_steps(20, 3)])
    eb = []
    for _ in range(6):
        b.run_sections(20)
        eb.append(b.thermo_energy())
    assert np.array_equal(ea, np.array(eb))
    for pa, pb in zip(a.download_paths(), b.download_paths()):
        assert np.array_equal(pa, pb)
    n0 = a.kernel_launches
    a.run_steps(20, 3, energies=False)
    assert a.kernel_launches - n0 == 9


@pytest.mark.parametrize("case", ["dot4_fn", "heg8", "dot2_small", "dot4_dr"])
@pytest.mark.parametrize("block,scratch_global,regs", [(64, 0, 4), (128, 1, 3), (256, 1, 2),
                                                       (256, 2, 3), (128, 2, 2),
                                                       (256, 0, 3), (512, 1, 1), (512, 0, 1)])
def test_launch_configs_match_golden(pimc, case, block, scratch_global, regs):
    # Every launch configuration the autotuner may pick reproduces pi-qmc's
    # decisions and action differences.
    g = golden_io.load(case)
    e = engine_for(pimc, g)
    fixed = any(g["kw"].get("node_kind", [0]))
    e.configure(block, scratch_global if fixed else 0, 0, regs)
    e.upload_paths([g["path0"]])
    n = min(g["nattempt"], 200)
    rec = e.run_sections(n, records=True)
    ref = g["records"]
    for k in ("ifirst1", "ipart", "reject_level"):
        assert np.array_equal(rec[k][0], ref[k][:n]), k
    nl = g["kw"]["nlevel"] + 1
    assert rel_close(rec["ds"][0][:, :nl], ref["ds"][:n, :nl], 1e-12)
    assert rel_close(rec["ds_node"][0][:, :nl], ref["ds_node"][:n, :nl], NODE_TOL.get(case, 1e-10))


@pytest.mark.parametrize("block,scratch_global,regs", [(64, 0, 2), (128, 0, 2), (256, 0, 2),
                                                       (512, 0, 1), (256, 1, 2), (256, 2, 2)])
def test_electron_gas_scratch_placements(pimc, block, scratch_global, regs):
    # 27 x 27 free-particle matrices: every shared-memory placement of the Slater
    # scratch (whole, hot part with the cold part and the new-column buffer in
    # global memory, all in global memory) reproduces pi-qmc's records.
    g = golden_io.load("heg54")
    e = engine_for(pimc, g)
    e.configure(block, scratch_global, 0, regs)
    e.upload_paths([g["path0"]])
    rec = e.run_sections(g["nattempt"], records=True)
    ref = g["records"]
    for k in ("ifirst1", "ipart", "reject_level"):
        assert np.array_equal(rec[k][0], ref[k]), k
    nl = g["kw"]["nlevel"] + 1
    assert rel_close(rec["ds"][0][:, :nl], ref["ds"][:, :nl], 1e-12)
    assert rel_close(rec["ds_node"][0][:, :nl], ref["ds_node"][:, :nl], 1e-10)
    assert np.abs(e.download_paths()[0] - g["path1"]).max() <= 1e-12


@pytest.mark.parametrize("case", ["dot2_small", "dot2_dr", "dot3_prim"])
@pytest.mark.parametrize("regs", [2, 4])
def test_one_warp_per_replica_matches_golden(pimc, case, regs):
    # Systems without node models may run one warp per replica (32-thread
    # blocks): pi-qmc's decisions, action differences and path all the same.
    g = golden_io.load(case)
    e = engine_for(pimc, g)
    e.configure(32, 0, 0, regs)
    assert e.launch_config()["block"] == 32
    e.upload_paths([g["path0"]])
    rec = e.run_sections(g["nattempt"], records=True)
    ref = g["records"]
    for k in ("ifirst1", "ipart", "reject_level"):
        assert np.array_equal(rec[k][0], ref[k]), k
    nl = g["kw"]["nlevel"] + 1
    assert rel_close(rec["ds"][0][:, :nl], ref["ds"][:, :nl], 1e-12)
    assert rel_close(rec["lnt"][0][:, :nl], ref["lnt"][:, :nl], 1e-12)
    assert np.abs(e.download_paths()[0] - g["path1"]).max() <= 1e-12


def test_one_warp_blocks_refused_with_node_models(pimc):
    g = golden_io.load("dot4_fn")
    e = engine_for(pimc, g)
    with pytest.raises(pimc.PimcError):
        e.configure(32, 0, 0, 2)


def test_autotune_does_not_advance_chains(pimc):
    g = golden_io.load("dot4_fn")
    a = engine_for(pimc, g, nreplica=8)
    b = engine_for(pimc, g, nreplica=8)
    for e in (a, b):
        e.upload_paths([g["path0"]] * 8)
    best, tried = a.autotune(8)
    assert len(tried) >= 3 and all(t["ms"] != 0 for t in tried)
    # the choice is one of the three fastest short trials (re-timed on longer ones)
    fastest = sorted((t for t in tried if t["ms"] > 0), key=lambda t: t["ms"])[:3]
    assert best["ms"] > 0 and any(t == best for t in fastest), (best, fastest)
    acc, att, st = a.replica_status()
    assert att.sum() == 0
    # the engine runs the shape the tuner reports (scratch placement included)
    applied = a.launch_config()
    assert all(applied[k] == best[k]
               for k in ("block", "scratch_global", "ctas_per_sm", "regs_variant")), (applied, best)
    b.configure(best["block"], best["scratch_global"], best["ctas_per_sm"], best["regs_variant"])
    ra = a.run_sections(40, records=True)
    rb = b.run_sections(40, records=True)
    assert np.array_equal(ra["reject_level"], rb["reject_level"])
    assert np.array_equal(ra["ds"], rb["ds"])
    for pa, pb in zip(a.download_paths(), b.download_paths()):
        assert np.array_equal(pa, pb)


def test_register_variants_bit_identical(pimc):
    # The register-budget variants compile the same arithmetic: same block size,
    # same results bit for bit.
    g = golden_io.load("dot4_fn")
    out = []
    for regs in (2, 3, 4, 1):
        e = engine_for(pimc, g, nreplica=4)
        e.configure(256, 0, 0, regs)
        e.upload_paths([g["path0"]] * 4)
        r = e.run_sections(60, records=True)
        out.append((r["ds"], r["ds_node"], r["reject_level"], e.download_paths(flat=True)))
    for o in out[1:]:
        for x, y in zip(out[0], o):
            assert np.array_equal(x, y)


@pytest.mark.parametrize("case", ["dot2_full", "dot4_fn", "heg8", "heg54", "dot20_fn"])
def test_estimators_match_golden(pimc, case):
    # Virial, Coulomb and optimized-Ewald Coulomb estimators through the ABI on
    # the final golden path against pi-qmc's own estimator values (the engine
    # sums pairs and windows in parallel: 1e-11 relative).
    g = golden_io.load(case)
    est = g["estimators"]
    e = engine_for(pimc, g, nreplica=2)
    e.upload_paths([g["path1"], g["path1"]])
    for w, v in est["virial"].items():
        got = e.virial_energy(w)
        assert np.allclose(got, v, rtol=1e-11, atol=1e-11), (w, got, v)
    assert np.allclose(e.coulomb_energy(1.0), est["coulomb"], rtol=1e-12)
    if "ewald" in est:
        x = est["ewald"]
        got = e.ewald_coulomb_energy(x["epsilon"], x["rcut"], x["table"], x["vgrid"])
        assert np.allclose(got, x["energy"], rtol=1e-11), (got, x["energy"])


@pytest.mark.parametrize("case", ["dot2_small", "dot2_full", "dot4_fn", "heg8"])
def test_displace_matches_golden(pimc, case):
    # Rigid displacement moves through the ABI from the final golden path, against
    # pi-qmc's DisplaceMoveSampler / DoubleDisplaceMoveSampler: particles,
    # displacements and decisions exact, action differences 1e-11 (the engine
    # sums slices and pairs in parallel), node terms 1e-9, final path 1e-12.
    g = golden_io.load(case)
    d = g["displace"]
    e = engine_for(pimc, g)
    e.upload_paths([g["path0"]])
    e.run_sections(g["nattempt"])  # the golden section attempts (path0 -> path1)
    assert d["first_attempt"] == g["nattempt"]
    r = e.run_displace(d["nattempt"], d["box"], d["nmoving"], d["species"], records=True)
    ref = d["records"]
    assert np.array_equal(r["ipart"][0], ref["ipart"])
    assert np.array_equal(r["disp"][0], ref["disp"])
    assert np.array_equal(r["accepted"][0], ref["accepted"])
    assert rel_close(r["ds"][0], ref["ds"], 1e-11)
    assert rel_close(r["ds_node"][0], ref["ds_node"], 1e-9)
    assert np.abs(e.download_paths()[0] - d["path"]).max() <= 1e-12


@pytest.mark.parametrize("case", ["dot4_fn", "dot2_full", "heg8", "heg16_hot", "dot20_fn",
                                  "dot2_dr", "dot4_dr"])
def test_mixed_form_on_identical_proposals(pimc, case):
    # Both precision forms draw the same FP64 proposals, so a mixed chain follows
    # the FP64 chain until a uniform falls within the mixed error of its
    # acceptance probability.  On the common attempts: ln T bit for bit (the
    # mover is FP64 in both), action differences (FP32 terms, compensated sums)
    # within 1e-4 of max(|dS|, 1), fixed-node differences (the mixed form
    # takes determinant ratios from cached inverses above level 0 and follows
    # moves by Sherman-Morrison updates between factorisations) within 1e-4 of
    # max(|dS_node|, 1) — 2e-3 on the ill-conditioned config-2 dot, its FP64
    # conditioning bar; the thermodynamic estimator on identical paths within
    # 1e-5 relative.
    g = golden_io.load(case)
    tol = NODE_TOL.get(case, 1e-4)
    n, R = (150, 8) if case != "dot20_fn" else (60, 4)
    out = []
    for prec in (1, 0):
        e = pimc.Engine(g["kw"], R, g["tables"], g["ewald"], seed=515, precision=prec)
        e.upload_paths([g["path0"]] * R)
        out.append((e, e.run_sections(n, records=True)))
    (em, m), (ef, f) = out
    same = np.ones(R, bool)
    compared = 0
    nl = g["kw"]["nlevel"] + 1
    for a in range(n):
        ok = ((m["reject_level"][:, a] == f["reject_level"][:, a]) &
              (m["ipart"][:, a] == f["ipart"][:, a]))
        for r in np.nonzero(same & ok)[0]:
            compared += 1
            lv = slice(0, nl)
            assert np.array_equal(m["lnt"][r, a, lv], f["lnt"][r, a, lv])
            fin = np.abs(f["ds"][r, a, lv]) < 1e99
            assert np.all(np.abs(m["ds"][r, a, lv] - f["ds"][r, a, lv])[fin]
                          <= 1e-4 * np.maximum(np.abs(f["ds"][r, a, lv][fin]), 1.0))
            fn = np.abs(f["ds_node"][r, a, lv]) < 1e99
            assert np.array_equal(np.abs(m["ds_node"][r, a, lv]) >= 1e99, ~fn)
            assert np.all(np.abs(m["ds_node"][r, a, lv] - f["ds_node"][r, a, lv])[fn]
                          <= tol * np.maximum(np.abs(f["ds_node"][r, a, lv][fn]), 1.0))
        same &= ok
    assert compared >= n * R // 2
    em.upload_paths(ef.download_paths())
    assert np.allclose(em.thermo_energy(), ef.thermo_energy(), rtol=1e-5, atol=0)
