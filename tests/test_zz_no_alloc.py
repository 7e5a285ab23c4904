"""The allocation-free node evaluation (pimc_node_evaluate_noalloc).

Callers that cannot allocate GPU memory — host code living inside another
framework's memory pool or budget, or a latency-critical loop that must not
call cudaMalloc/cudaFree — evaluate Slater determinants and nodal distances
through this entry point on their own device buffers; its scratch is a fixed
static device array.  This file is collected last on purpose: it checks the
entry point through the C ABI against the engine's pimc_node_evaluate on the
same inputs, twice in a row (the second call reuses the shared scratch left by
the first).  Both kernels run the same warp-level Slater evaluation
(node_eval_warp) on the same inputs; only where the scratch lives (a static
global array here, shared memory there) differs, so the results must agree bit
for bit.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CASES = {
    # SHONodes with 10 particles per species at a temperature where the Slater
    # matrices are well conditioned, and FreeParticleNodes in a periodic box.
    "sho10": dict(counts=[10, 10], sho_omega=[1.0, 1.0], nslice=64, beta=2.0, nlevel=3,
                  node_kind=[1, 1], node_omega=[1.0, 1.0], cell=1000.0),
    "free4": dict(counts=[4, 4], nslice=128, beta=17.376, nlevel=3, node_kind=[2, 2],
                  cell=12.895, mover=1),
}


@pytest.mark.parametrize("case", list(CASES))
def test_noalloc_matches_engine_node_evaluate(case):
    import torch

    import pimc_gb300
    pimc_gb300.build.build()
    kw = CASES[case]
    eng = pimc_gb300.Engine(kw, 1)
    npart = sum(kw["counts"])
    rng = np.random.default_rng(11)
    nb = 200  # more entries than scratch slots: the grid-stride loop reuses them
    spread = 1.0 if case == "sho10" else kw["cell"] / 3
    r1 = spread * rng.normal(size=(nb, npart, 3))
    r2 = r1 + 0.3 * rng.normal(size=(nb, npart, 3))
    sysc = pimc_gb300.system_from_kw(kw)
    L = pimc_gb300.lib()
    dev = torch.device("cuda:0")
    t1 = torch.from_numpy(r1).to(dev)
    t2 = torch.from_numpy(r2).to(dev)
    for sp in range(2):
        err, det, d1, d2 = eng.node_evaluate(sp, r1, r2)
        scale = eng.node_scale(0, sp)
        for call in range(2):
            odet = torch.full((nb,), float("nan"), dtype=torch.float64, device=dev)
            od1 = torch.full((nb, npart), float("nan"), dtype=torch.float64, device=dev)
            od2 = torch.full((nb, npart), float("nan"), dtype=torch.float64, device=dev)
            oerr = torch.full((nb,), -1, dtype=torch.int32, device=dev)
            stream = torch.cuda.current_stream().cuda_stream
            rc = L.pimc_node_evaluate_noalloc(
                C.byref(sysc), sp, scale, nb, C.c_void_p(t1.data_ptr()),
                C.c_void_p(t2.data_ptr()), C.c_void_p(odet.data_ptr()),
                C.c_void_p(od1.data_ptr()), C.c_void_p(od2.data_ptr()),
                C.c_void_p(oerr.data_ptr()), C.c_void_p(stream))
            assert rc == 0, L.pimc_last_error().decode()
            torch.cuda.synchronize()
            assert np.array_equal(oerr.cpu().numpy(), err), (sp, call)
            assert np.array_equal(odet.cpu().numpy(), det), (sp, call)
            assert np.array_equal(od1.cpu().numpy(), d1), (sp, call)
            assert np.array_equal(od2.cpu().numpy(), d2), (sp, call)


def test_noalloc_rejects_oversized_species():
    # A 33-particle species is refused before any launch.  The buffers are real
    # device allocations of the sizes the call names, so that even a wrongly
    # accepted call would only touch memory it owns.
    import torch

    import pimc_gb300
    pimc_gb300.build.build()
    kw = dict(counts=[33], nslice=64, beta=2.0, nlevel=3, node_kind=[1], node_omega=[1.0],
              sho_omega=[1.0], cell=1000.0)
    sysc = pimc_gb300.system_from_kw(kw)
    dev = torch.device("cuda:0")
    pos = torch.zeros((33, 3), dtype=torch.float64, device=dev)
    det = torch.zeros((1,), dtype=torch.float64, device=dev)
    dist = torch.zeros((2, 33), dtype=torch.float64, device=dev)
    err = torch.zeros((1,), dtype=torch.int32, device=dev)
    p = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731
    rc = pimc_gb300.lib().pimc_node_evaluate_noalloc(
        C.byref(sysc), 0, 1.0, 1, p(pos), p(pos), p(det), p(dist[0]), p(dist[1]), p(err), None)
    torch.cuda.synchronize()
    assert rc != 0
    assert "32" in pimc_gb300.lib().pimc_last_error().decode()
    assert not torch.any(det != 0) and not torch.any(err != 0)
