"""The CPU checkers: the restatement (oracle/port.cc) pinned against pi-qmc's
own unit-test known answers, the golden fixtures made by pi-qmc's own code,
and (where the reference tree is present) oracle/_ref directly."""
import ctypes as C
import os

import numpy as np
import pytest

import golden_io
import oracle_lib as O
import workloads as W

# Tolerances.  Plain action differences and mover ratios: 1e-12 relative.
# Node-model differences: 1e-10 relative for well-conditioned Slater matrices.
# dot20_fn (SHONodes at omega/T = 20) is the exception: its 10x10 Slater
# matrices have 1-norm condition numbers of 1e12 - 3e13 (tests/golden/nodes_dot20_fn.npz,
# computed in 60-digit arithmetic), and rounding the matrix elements to FP64
# alone, before any factorisation, moves the determinant by up to 3e-5.  Against
# the 60-digit values of the same double inputs, pi-qmc (OpenBLAS dgetrf/dgetri)
# lands within 1.1e-3 and this restatement within 9e-4 on determinants and
# nodal distances, and the two differ from each other by up to 6e-4.  That case
# is held to 2e-3 relative on node values and nodal action, with exact decisions.
NODE_TOL = {"dot20_fn": 2e-3}
EXACT_TOL = 2e-3   # FP64 against the 60-digit values, for the ill-conditioned dot


def rel_close(a, b, tol, floor=1.0):
    return np.all(np.abs(a - b) <= tol * np.maximum(np.abs(a), floor))


def port_for(case):
    g = golden_io.load(case)
    cfg = O.make_config(**g["kw"])
    return g, cfg, O.PortOracle(cfg, g["tables"], g["ewald"])


# ---- reference unit-test known answers -----------------------------------
def _lib():
    return O.PortOracle.lib()


def test_sho_action_known_answer():
    # unit-tests/action/SHOActionTest.cc:62-70: one bead of 64 moved to (1,2,3).
    cfg = O.make_config(counts=[1], sho_omega=[1.0], nslice=64, beta=6.4, nlevel=6,
                        spring=0, cell=10.0)
    sec = np.zeros((65, 1, 3))
    mov = np.zeros((65, 1, 3))
    assert O.PortOracle(cfg).action_diff(0, sec, mov, 0) == 0.0
    mov[32, 0] = [1, 2, 3]
    d = O.PortOracle(cfg).action_diff(0, sec, mov, 0)
    assert np.float32(d) == pytest.approx(np.float32(0.46635586), rel=4 * 2.0 ** -23)


@pytest.mark.parametrize("a,b", [(0.5, 0.0), (0.5, 1.0)])
def test_prim_sho_known_answer(a, b):
    # unit-tests/action/PrimSHOActionTest.cc:56-79: (a r^2 + b r^4) tau.
    cfg = O.make_config(counts=[1], prim_a=[a], prim_b=[b], nslice=64, beta=6.4,
                        nlevel=6, spring=0, cell=10.0)
    sec = np.zeros((65, 1, 3))
    mov = np.zeros((65, 1, 3))
    mov[32, 0] = [1, 2, 3]
    r2 = 14.0
    d = O.PortOracle(cfg).action_diff(0, sec, mov, 0)
    assert np.float32(d) == pytest.approx(np.float32((a * r2 + b * r2 * r2) * 0.1),
                                          rel=4 * 2.0 ** -23)


def test_periodic_gaussian_known_answers():
    # unit-tests/util/PeriodicGaussianTest.cc:24-92 (alpha=2.5, L=1.5).
    L = _lib()
    L.port_pg_terms.restype = C.c_int
    L.port_pg_terms.argtypes = [C.c_double, C.c_double]
    L.port_pg_eval.restype = C.c_double
    L.port_pg_eval.argtypes = [C.c_double, C.c_double, C.c_double, C.POINTER(C.c_double)]
    assert L.port_pg_terms(2.5, 1.5) == 5
    assert L.port_pg_terms(2.5, 20.0) == 64
    g = C.c_double()
    for x, v, dv in [(0.0, 1.0072131266104112, 0.0),
                     (0.4999 * 1.5, 0.49012750361989998, -0.00066637454689608252),
                     (-0.3 * 1.5, 0.66635569537953232, 1.0233852136355668)]:
        val = L.port_pg_eval(2.5, 1.5, x, C.byref(g))
        assert val == pytest.approx(v, rel=4e-16, abs=0)
        assert g.value == pytest.approx(dv, rel=1e-14, abs=1e-15)


def test_supercell_pbc_known_answer():
    # unit-tests/util/SuperCellTest.cc:12-32.
    L = _lib()
    L.port_pbc.argtypes = [C.POINTER(C.c_double), C.POINTER(C.c_double)]
    a = (C.c_double * 3)(1, 2, 4)
    v = (C.c_double * 3)(0.1, 2, 2.5)
    L.port_pbc(a, v)
    assert list(v) == [0.1, 0.0, -1.5]


# ---- golden fixtures from pi-qmc's own code ---------------------------------
@pytest.mark.parametrize("case", list(W.GOLDEN_CASES))
def test_port_matches_golden(case):
    g, cfg, port = port_for(case)
    port.set_path(g["path0"])
    assert port.thermo_energy() == pytest.approx(g["energy0"], rel=1e-12)
    r = port.run(g["nattempt"])
    ref = g["records"]
    for k in ("ifirst1", "ifirst2", "ipart", "reject_level"):
        assert np.array_equal(r[k], ref[k]), k
    assert r["naccepted"] == g["naccepted"]
    assert rel_close(r["ds"], ref["ds"], 1e-12)
    assert rel_close(r["lnt"], ref["lnt"], 1e-12)
    assert rel_close(r["ds_node"], ref["ds_node"], NODE_TOL.get(case, 1e-10))
    assert np.abs(port.get_path() - g["path1"]).max() <= 1e-12
    assert port.thermo_energy() == pytest.approx(g["energy1"], rel=1e-12)


# ---- direct comparison with the reference build (where it exists) ---------
needs_ref = pytest.mark.skipif(not O.RefOracle.available(),
                               reason="oracle/_ref not built (no reference tree)")


@needs_ref
@pytest.mark.parametrize("seed", [11, 12, 13])
def test_port_matches_reference_dot(seed):
    kw = W.dot2(nslice=128, seed=seed)
    cfg = O.make_config(**kw)
    ref = O.RefOracle(cfg)
    port = O.PortOracle(cfg, ref.pair_tables(), ref.ewald_table())
    x = W.initial_path(cfg, "gauss", seed=seed)
    ref.set_path(x)
    port.set_path(x)
    a, b = ref.run(500), port.run(500)
    for k in ("ifirst1", "ipart", "reject_level"):
        assert np.array_equal(a[k], b[k])
    assert rel_close(a["ds"], b["ds"], 1e-12)
    assert np.array_equal(ref.get_path(), port.get_path())


@needs_ref
@pytest.mark.parametrize("factors", [(0.0, 0.0), (0.8, 0.5), (1.4, 1.1)])
@pytest.mark.parametrize("fixed", [False, True])
def test_port_matches_reference_delayed_rejection(factors, fixed):
    # Delayed rejection (MultiLevelSampler / DoubleMLSampler with the
    # FreeMover) at pi-qmc's default and at other sigma factors, the
    # restatement against pi-qmc's own code on the same streams.
    sf, nf = factors
    if fixed:
        kw = W.dot20_fn(counts=[2, 2], nslice=64, beta=4.0, nlevel=3, seed=21)
        init = "const"
    else:
        kw = W.dot2(nslice=64, seed=21)
        init = "gauss"
    kw = dict(kw, delayed_rejection=1, sigma_factor=sf, dr_sigma_factor=nf)
    cfg = O.make_config(**kw)
    ref = O.RefOracle(cfg)
    port = O.PortOracle(cfg, ref.pair_tables(), ref.ewald_table())
    x = W.initial_path(cfg, init, seed=21)
    ref.set_path(x)
    port.set_path(x)
    a, b = ref.run(300), port.run(300)
    for k in ("ifirst1", "ipart", "reject_level"):
        assert np.array_equal(a[k], b[k]), k
    assert rel_close(a["ds"], b["ds"], 1e-12)
    assert rel_close(a["lnt"], b["lnt"], 1e-12)
    assert np.abs(ref.get_path() - port.get_path()).max() <= 1e-12


@needs_ref
def test_port_matches_reference_action_levels():
    # Action-level parity at every level on random sections (FakeSampler).
    kw = W.dot20_fn(counts=[3, 2], nslice=64, nlevel=4, node_kind=[0, 0])
    cfg = O.make_config(**kw)
    ref = O.RefOracle(cfg)
    port = O.PortOracle(cfg, ref.pair_tables(), None)
    rng = np.random.default_rng(5)
    for trial in range(20):
        sec = rng.normal(size=(17, 5, 3))
        ip = int(rng.integers(5))
        mov = sec[:, ip, :].copy()
        mov[1:-1] += 0.3 * rng.normal(size=(15, 3))
        for level in range(5):
            a = ref.action_diff(level, sec, mov, ip)
            b = port.action_diff(level, sec, mov, ip)
            assert abs(a - b) <= 1e-12 * max(abs(a), 1.0)


@pytest.mark.parametrize("case", list(W.GOLDEN_CASES))
def test_port_estimators_match_golden(case):
    # Virial (windows 1, 4, 16), direct Coulomb and optimized-Ewald Coulomb
    # estimators of the restatement on the final golden path against the values
    # pi-qmc's own estimator classes produced.
    g = golden_io.load(case)
    est = g["estimators"]
    port = O.PortOracle(O.make_config(**g["kw"]), g["tables"], g["ewald"])
    port.set_path(g["path1"])
    for w, v in est["virial"].items():
        assert port.virial_energy(w) == pytest.approx(v, rel=1e-12, abs=1e-12), w
    assert est["virial"][1] == pytest.approx(g["energy1"], rel=1e-12)  # window 1 = thermo
    assert port.coulomb_energy(1.0) == pytest.approx(est["coulomb"], rel=1e-13)
    if "ewald" in est:
        e = est["ewald"]
        got = port.ewald_coulomb_energy(e["epsilon"], e["rcut"], e["table"], e["vgrid"])
        assert got == pytest.approx(e["energy"], rel=1e-12)


def test_estimator_ewald_builder_against_reference():
    # The engine's own optimized-Ewald fit for the estimator: same k-list as
    # pi-qmc's, coefficients set by a differently conditioned solve, so the
    # tables agree to ~1e-3 and the energy to ~2e-4 (pi-qmc's coefficients are
    # themselves rounding-determined for this system).
    import pimc_gb300
    g = golden_io.load("heg8")
    e = g["estimators"]["ewald"]
    ew, vg = pimc_gb300.ewald_estimator_tables(g["kw"], e["rcut"], e["kcut"], e["epsilon"])
    assert ew["totk"] == e["table"]["totk"]
    assert np.array_equal(ew["kvec"], e["table"]["kvec"])
    assert np.max(np.abs(ew["vk"] - e["table"]["vk"])) <= 5e-3 * np.abs(e["table"]["vk"]).max()
    assert np.max(np.abs(vg - e["vgrid"])) <= 5e-3 * np.abs(e["vgrid"]).max()
    port = O.PortOracle(O.make_config(**g["kw"]), g["tables"], g["ewald"])
    port.set_path(g["path1"])
    got = port.ewald_coulomb_energy(e["epsilon"], e["rcut"], ew, vg)
    assert got == pytest.approx(e["energy"], rel=1e-3)


@pytest.mark.parametrize("case", ["dot2_small", "dot2_full", "dot4_fn", "heg8"])
def test_port_displace_matches_golden(case):
    # Rigid displacement moves (DisplaceMoveSampler / DoubleDisplaceMoveSampler)
    # from the final golden path: particles, displacements and decisions exact,
    # action differences 1e-12 (node terms 1e-10), final path 1e-12.
    g = golden_io.load(case)
    d = g["displace"]
    port = O.PortOracle(O.make_config(**g["kw"]), g["tables"], g["ewald"])
    port.set_path(g["path1"])
    r = port.run_displace(d["nattempt"], d["box"], d["nmoving"], d["species"],
                          first_attempt=d["first_attempt"])
    ref = d["records"]
    assert np.array_equal(r["ipart"], ref["ipart"])
    assert np.array_equal(r["accepted"], ref["accepted"])
    assert np.array_equal(r["disp"], ref["disp"])
    assert np.allclose(r["ds"], ref["ds"], rtol=1e-12, atol=1e-12)
    assert np.allclose(r["ds_node"], ref["ds_node"], rtol=1e-10, atol=1e-10)
    assert np.abs(port.get_path() - d["path"]).max() <= 1e-12


@pytest.mark.parametrize("case", list(W.NODE_CASES))
def test_port_node_models_match_golden(case):
    # SHONodes / FreeParticleNodes of the restatement on pi-qmc's own
    # NodeModel::evaluate + evaluateDistance outputs (same slice pairs, same
    # scale): determinant, error flag and both distance arrays.  For the
    # ill-conditioned dot both are also held to the 60-digit values.
    z = golden_io.load_nodes(case)
    g = golden_io.load(case)
    cfg = O.make_config(**z["kw"])
    port = O.PortOracle(cfg, g["tables"], g["ewald"])
    tol = NODE_TOL.get(case, 1e-12)
    nb = len(z["r1"])
    assert z["species"], case
    for sp, ref in z["species"].items():
        O.PortOracle.lib().port_set_node_scale(port.h, sp, ref["scale"])
        for b in range(nb):
            err, det, d1, d2 = port.node_eval(sp, z["r1"][b], z["r2"][b], 0, False)
            assert err == ref["err"][b]
            assert abs(det - ref["det"][b]) <= tol * abs(ref["det"][b]), (sp, b)
            assert rel_close(d1, ref["d1"][b], tol, floor=0.0), (sp, b)
            assert rel_close(d2, ref["d2"][b], tol, floor=0.0), (sp, b)
            if "exact_det" in ref:
                f, n = ref["first"], cfg.spec_count[sp]
                for got in (det, ref["det"][b]):
                    assert abs(got - ref["exact_det"][b]) <= EXACT_TOL * abs(ref["exact_det"][b])
                for got, ex in ((d1, ref["exact_d1"][b]), (d2, ref["exact_d2"][b]),
                                (ref["d1"][b], ref["exact_d1"][b]),
                                (ref["d2"][b], ref["exact_d2"][b])):
                    assert rel_close(got[f:f + n], ex, EXACT_TOL, floor=0.0), (sp, b)


def test_node_fixtures_exercise_the_nodal_action():
    # The periodic golden cases are not vacuous: pi-qmc's records of the warm
    # electron gas hold nonzero free-particle nodal actions and node crossings
    # (2e100), and the other cases' dot and gas node terms are nonzero too.
    g = golden_io.load("heg16_hot")
    dsn = g["records"]["ds_node"][:, :g["kw"]["nlevel"] + 1]
    assert np.sum((dsn != 0) & (dsn < 1e99)) > 500
    assert np.sum(dsn >= 1e99) >= 3
    for case in W.NODE_CASES:
        for ref in golden_io.load_nodes(case)["species"].values():
            assert np.all(ref["det"] != 0) and np.all(np.isfinite(ref["d1"]))
            assert np.any(ref["d1"] < 200) and np.any(ref["d2"] < 200)


def test_oracle_structs_match_the_header(tmp_path):
    # The ctypes structures of oracle_lib have oracle_api.h's layouts.
    import ctypes as C
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    hdr = os.path.join(os.path.dirname(O.__file__), "oracle_api.h")
    structs = {"ora_config": O.OraConfig, "ora_record": O.OraRecord,
               "ora_drecord": O.OraDRecord, "ora_pair_table": O.OraPairTable,
               "ora_ewald_table": O.OraEwaldTable}
    lines = ["#include <stdio.h>", "#include <stddef.h>", "#include <stdint.h>",
             f'#include "{hdr}"', "int main(void) {"]
    for cname, cls in structs.items():
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in cls._fields_:
            lines.append(f'  printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-std=c99", str(src), "-o", str(exe)], check=True)
    got = {}
    for line in subprocess.run([str(exe)], capture_output=True, text=True,
                               check=True).stdout.split("\n"):
        if line:
            a, b, v = line.split()
            got[(a, b)] = int(v)
    for cname, cls in structs.items():
        assert got[(cname, "size")] == C.sizeof(cls), cname
        for fname, _ in cls._fields_:
            assert got[(cname, fname)] == getattr(cls, fname).offset, (cname, fname)

