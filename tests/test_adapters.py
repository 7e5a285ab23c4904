"""The pi-qmc-side adapters (pi-qmc_gb300/adapters) compile against pi-qmc's
own headers and, linked with pi-qmc's objects and a stand-in of the engine's C
ABI (computed by the CPU restatement), run inside pi-qmc's own samplers and
reproduce pi-qmc's golden records; checked wherever the reference tree exists."""
import ctypes as C
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


def _write_input(fname, g, n):
    import numpy as np

    import oracle_lib as O
    cfg = O.make_config(**g["kw"])
    with open(fname, "wb") as f:
        f.write(bytes(cfg))
        f.write(np.int32(len(g["tables"])).tobytes())
        for t in g["tables"]:
            s1, s2 = t["species"]
            f.write(np.array([s1, s2, t["ngpts"], t["norder"]], np.int32).tobytes())
            f.write(np.array([t["rgridinv"], t["logrratioinv"]]).tobytes())
            f.write(np.ascontiguousarray(t["ugrid"], np.float64).tobytes())
        ew = g["ewald"]
        f.write(np.int32(ew is not None).tobytes())
        if ew is not None:
            f.write(np.int32(ew["totk"]).tobytes())
            f.write(np.ascontiguousarray(ew["kvec"], np.int32).tobytes())
            f.write(np.ascontiguousarray(ew["vk"], np.float64).tobytes())
            f.write(np.array([ew["one_over_2v"], ew["self_energy"]]).tobytes())
            f.write(np.array(ew["ikmax"], np.int32).tobytes())
        f.write(np.ascontiguousarray(g["path0"], np.float64).tobytes())
        f.write(np.int32(n).tobytes())
    return cfg


@pytest.fixture(scope="module")
def adapter_check(tmp_path_factory):
    """pi-qmc's objects + the adapters + a stand-in of the engine's C ABI
    computed by the CPU restatement, linked into one program."""
    if not (os.path.isdir(os.path.join(REF, "src")) and
            os.path.exists(os.path.join(REPO, "oracle", "_ref", "libpimcref.so"))):
        pytest.skip("pi-qmc source tree and its compiled objects not present")
    import oracle_lib
    port = oracle_lib.build_port()
    refdir = os.path.join(REPO, "oracle", "_ref")
    exe = str(tmp_path_factory.mktemp("adapters") / "adapter_check")
    cmd = ["g++", "-std=gnu++11", "-O1", "-w", "-DHAVE_CONFIG_H", "-ffp-contract=off",
           "-I" + os.path.join(REPO, "oracle", "shim"), "-I" + os.path.join(REF, "src"),
           "-I" + os.path.join(REF, "contrib", "blitz-0.9"),
           "-I" + os.path.join(REPO, "include"), "-I" + os.path.join(REPO, "oracle"),
           "-I" + os.path.join(REPO, "pi-qmc_gb300", "adapters"),
           os.path.join(REPO, "tests", "adapters", "adapter_check.cc"),
           os.path.join(REPO, "tests", "adapters", "standin_engine.cc"),
           os.path.join(REPO, "pi-qmc_gb300", "adapters", "GpuAdapters.cc"), "-o", exe,
           "-L" + refdir, "-lpimcref", "-Wl,-rpath," + refdir, port,
           "-Wl,-rpath," + os.path.dirname(port)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr[-3000:]
    return exe


@pytest.mark.parametrize("case,n", [("dot4_fn", 200), ("dot20_fn", 40), ("heg8", 100),
                                    ("dot3_prim", 200)])
def test_adapters_reproduce_golden_records(adapter_check, tmp_path, case, n):
    # pi-qmc's own DoubleMLSampler + FixedNodeAction(GpuNodeModel) and
    # MultiLevelSampler + GpuCompositeAction reproduce the records pi-qmc made
    # with its own actions and node models; GpuSectionSampler and
    # gpuThermoEnergy on pi-qmc's Paths reproduce its final path and energy.
    import numpy as np

    import golden_io
    import oracle_lib as O
    g = golden_io.load(case)
    inp, outp = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    cfg = _write_input(inp, g, n)
    r = subprocess.run([adapter_check, inp, outp], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    raw = open(outp, "rb").read()
    rs = C.sizeof(O.OraRecord)
    recs = O.records_to_numpy((O.OraRecord * n).from_buffer_copy(raw[:n * rs]), n)
    np_path = cfg.nslice * cfg.npart * 3
    path1 = np.frombuffer(raw[n * rs:n * rs + 8 * np_path]).reshape(cfg.nslice, cfg.npart, 3)
    energy = np.frombuffer(raw[n * rs + 8 * np_path:n * rs + 8 * np_path + 8])[0]
    counts = np.frombuffer(raw[n * rs + 8 * np_path + 8:], np.int32)
    ref = g["records"]
    for k in ("ifirst1", "ifirst2", "ipart", "reject_level"):
        assert np.array_equal(recs[k], ref[k][:n]), k
    tol = 2e-3 if case == "dot20_fn" else 1e-10
    floor = np.maximum(np.abs(ref["ds"][:n]), 1.0)
    assert np.all(np.abs(recs["ds"] - ref["ds"][:n]) <= 1e-12 * floor)
    fl = np.maximum(np.abs(ref["ds_node"][:n]), 1.0)
    assert np.all(np.abs(recs["ds_node"] - ref["ds_node"][:n]) <= tol * fl)
    fixed = any(g["kw"].get("node_kind", [0]))
    assert counts[1] > 0 and (counts[0] > 0) == fixed
    if n == g["nattempt"]:
        assert np.abs(path1 - g["path1"]).max() <= 1e-12
        assert energy == pytest.approx(g["energy1"], rel=1e-12)
    if case == "dot20_fn":
        assert counts[2] > 0  # pi-qmc's set-up rescaled the determinant: the scale followed


def test_gpu_tags_parse_into_the_engine_system(tmp_path):
    """<GpuAction> with pi-qmc's own action children (SpringAction, SHOAction,
    PrimSHOAction, CoulombAction, FixedNodeAction with SHONodes) parsed by the
    GPU tag parser on pi-qmc's XMLParser (compiled from the reference tree,
    libxml2 replaced by a stand-in) into the engine's system; unknown tags and
    a sampler mover that disagrees are refused; <GpuSample> builds the device
    sampler."""
    if not (os.path.isdir(os.path.join(REF, "src")) and
            os.path.exists(os.path.join(REPO, "oracle", "_ref", "libpimcref.so"))):
        pytest.skip("pi-qmc source tree and its compiled objects not present")
    import oracle_lib
    port = oracle_lib.build_port()
    refdir = os.path.join(REPO, "oracle", "_ref")
    exe = str(tmp_path / "parser_check")
    cmd = ["g++", "-std=gnu++11", "-O1", "-w", "-DHAVE_CONFIG_H",
           "-I" + os.path.join(REPO, "tests", "adapters", "stub_libxml"),
           "-I" + os.path.join(REPO, "oracle", "shim"), "-I" + os.path.join(REF, "src"),
           "-I" + os.path.join(REF, "contrib", "blitz-0.9"),
           "-I" + os.path.join(REPO, "include"), "-I" + os.path.join(REPO, "oracle"),
           "-I" + os.path.join(REPO, "pi-qmc_gb300", "adapters"),
           os.path.join(REPO, "tests", "adapters", "parser_check.cc"),
           os.path.join(REPO, "pi-qmc_gb300", "adapters", "GpuParser.cc"),
           os.path.join(REPO, "pi-qmc_gb300", "adapters", "GpuAdapters.cc"),
           os.path.join(REPO, "tests", "adapters", "standin_engine.cc"),
           os.path.join(REF, "src", "parser", "XMLParser.cc"), "-o", exe,
           "-L" + refdir, "-lpimcref", "-Wl,-rpath," + refdir, port,
           "-Wl,-rpath," + os.path.dirname(port)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr[-3000:]
    out = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert out.returncode == 0, out.stderr
    lines = [l for l in out.stdout.splitlines() if l and l[0].isdigit()]
    v = lines[-4].split()
    # npart nspecies counts sho_omega prim_a prim_a prim_b mass charge cell node_kind
    # node_omega node_temperature nslice tau nlevel epsilon spring coulomb norder mover replicas
    assert v[:12] == ["4", "2", "2", "2", "1", "1", "0", "0.5", "0.25", "1", "-1", "1000"]
    assert v[12:17] == ["1", "1", "1.25", "1.5", "0.5"]
    assert v[17] == "64" and float(v[18]) == 4.0 / 64 and v[19] == "3"
    assert v[20:26] == ["2", "1", "1", "3", "0", "7"]
    assert lines[-3] == "1"              # precision: mixed
    # delayedRejection, defaultSigmaFactor (0: pi-qmc's default), newSigmaFactor
    assert lines[-2] == "1 0 0.6"
    assert lines[-1] == "3 1"            # the three refusals, and a sampler
