"""Serving engine on the GPU: slots over one device pool, continuous batching.

* a simulation served in a slot follows exactly the chain of the same system
  run as replica 0 of a plain engine (same kernels, stream id 0);
* a request's final path and energy samples are bit-identical whether it is
  served alone or in a mix of requests that arrive, run and leave around it;
* the pool admits by its byte budget, refuses when full and reuses freed space.
"""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "..", "pi-qmc_gb300"))
import pimc_gb300  # noqa: E402
from pimc_gb300 import serving  # noqa: E402
from pimc_gb300 import workloads as W  # noqa: E402

pytestmark = pytest.mark.gpu
SEED = 777


def small_dot(n_up, n_dn, m, lev, w):
    counts = [n_up, n_dn]
    return dict(counts=counts, sho_omega=[w, w], nslice=m, beta=m / 25.6, nlevel=lev,
                coulomb=1, norder=3, node_kind=[1, 1], node_omega=[w, w],
                node_temperature=w / 4.0, cell=W.DOT_CELL)


@pytest.fixture(scope="module")
def base_tables():
    kw = small_dot(2, 2, 128, 4, 1.0)
    tabs, _ = pimc_gb300.coulomb_tables(kw)
    return tabs


def path_for(kw, seed):
    return W.initial_path(kw, "const", seed=seed) * (1.0 / np.sqrt(kw["sho_omega"][0]))


def test_server_slot_follows_engine_replica(base_tables):
    kw = small_dot(3, 2, 128, 4, 1.2)
    tabs = W.tables_for(kw, base_tables)
    p0 = path_for(kw, 3)
    eng = pimc_gb300.Engine(kw, 1, tabs, None, seed=SEED)
    eng.upload_paths([p0])
    srv = pimc_gb300.Server(4, 64 << 20, 64, 2048, 5, 32, seed=SEED)
    slot = srv.admit(kw, tabs, p0, 0, 32)
    assert slot is not None
    for _ in range(6):
        eng.run_sections(32)
        srv.run()
        e1 = eng.thermo_energy()[0]
        e2 = srv.energies()[slot]
        assert abs(e1 - e2) <= 1e-12 * abs(e1)
        assert srv.energies([slot])[0] == e2  # measuring a subset gives the same value
    assert np.array_equal(eng.download_paths()[0], srv.download_path(slot))
    acc, att, st = srv.replica_status()
    assert att[slot] == 6 * 32 and st[slot] == 0


def make_requests(base_tables, n, seed):
    out = []
    for i, (t, kw, sw) in enumerate(W.serve_stream(n, rate=2000.0, seed=seed, nmax=24,
                                                   slices=(64, 128, 256), sweep_scale=1e-4)):
        att = max(8, int(sw * W.sweep_attempts(kw)))
        out.append(serving.Request(i, kw, W.tables_for(kw, base_tables), path_for(kw, 100 + i),
                                   att, t))
    return out


def test_same_result_alone_and_in_mix(base_tables):
    reqs = make_requests(base_tables, 24, seed=11)
    budget = serving.DEFAULT_ROUND_BUDGET / 8
    srv = pimc_gb300.Server(6, 16 << 20, 64, 2048, 5, 32, seed=SEED)
    loop = serving.ServeLoop(srv, round_budget=budget, keep_paths=True)
    loop.run(reqs, realtime=False)
    assert loop.overlapped > 0  # requests were admitted while others ran
    used, _ = srv.pool()
    assert used == 0
    for k in (0, 5, 13, 23):
        alone = make_requests(base_tables, 24, seed=11)[k]
        solo = pimc_gb300.Server(6, 16 << 20, 64, 2048, 5, 32, seed=SEED)
        serving.ServeLoop(solo, round_budget=budget, keep_paths=True).run([alone],
                                                                         realtime=False)
        assert alone.round_attempts == reqs[k].round_attempts
        assert len(alone.energies) == len(reqs[k].energies), k
        assert np.all(np.isfinite(alone.energies)), k
        assert np.array_equal(alone.final_path, reqs[k].final_path), k
        assert alone.energies == reqs[k].energies, k


def test_pool_budget(base_tables):
    kw = small_dot(4, 4, 256, 5, 1.0)
    tabs = W.tables_for(kw, base_tables)
    p = path_for(kw, 1)
    path_bytes = p.nbytes
    srv = pimc_gb300.Server(16, 3 * path_bytes + path_bytes // 2, 64, 2048, 5, 32, seed=SEED)
    # each admission holds the path plus its Slater-result cache, so fewer than 3 fit
    slots = []
    while True:
        s = srv.admit(kw, tabs, p, len(slots), 16)
        if s is None:
            break
        slots.append(s)
    assert 1 <= len(slots) < 3
    used, big = srv.pool()
    assert used > 0 and big < used / len(slots)
    srv.release(slots[0])
    assert srv.admit(kw, tabs, p, 99, 16) == slots[0]
    with pytest.raises(pimc_gb300.PimcError):  # beyond the server's maxima: never admissible
        srv.admit(small_dot(40, 40, 256, 5, 1.0), tabs, np.zeros((256, 80, 3)), 5, 16)
