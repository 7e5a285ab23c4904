"""Host logic of the serving loop (continuous batching), on a fake server.

The fake keeps the real server's contract: a fixed number of slots, a byte
budget for paths, admit() returning None when either is exhausted, and energies
that depend only on a simulation's own id and progress.  The loop must admit by
budget, never exceed it, finish every request, and give each request the same
samples alone and in a mix.
"""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "..", "pi-qmc_gb300"))
from pimc_gb300 import serving  # noqa: E402
from pimc_gb300 import workloads as W  # noqa: E402


class FakeServer:
    def __init__(self, slots, budget):
        self.slots, self.budget = slots, budget
        self.used = 0
        self.live = {}
        self.max_live = 0
        self.max_used = 0

    def admit(self, kw, tables, path, rid, round_attempts):
        nbytes = path.nbytes
        free = [s for s in range(self.slots) if s not in self.live]
        if not free or self.used + nbytes > self.budget:
            return None
        s = free[0]
        self.live[s] = [rid, 0, nbytes, round_attempts]
        self.used += nbytes
        self.max_live = max(self.max_live, len(self.live))
        self.max_used = max(self.max_used, self.used)
        return s

    def release(self, s):
        self.used -= self.live.pop(s)[2]

    def run(self):
        for v in self.live.values():
            v[1] += v[3]

    def energies(self, slots=None):
        e = np.full(self.slots, np.nan)
        for s, (rid, att, _, _) in self.live.items():
            e[s] = np.sin(rid * 1.3 + att * 0.01)
        return e if slots is None else e[list(slots)]

    def download_path(self, s):
        return np.zeros(1)


def make_requests(n, seed=5):
    out = []
    for i, (t, kw, sw) in enumerate(W.serve_stream(n, rate=1e5, seed=seed, sweep_scale=1e-3)):
        path = np.zeros((kw["nslice"], sum(kw["counts"]), 3))
        out.append(serving.Request(i, kw, [], path, int(sw * W.sweep_attempts(kw)) + 1, t))
    return out


def test_stream_shapes():
    s = W.serve_stream(400, seed=1)
    ns = [sum(kw["counts"]) for _, kw, _ in s]
    ms = {kw["nslice"] for _, kw, _ in s}
    assert min(ns) >= 2 and max(ns) <= 64 and len(set(ns)) > 40
    assert ms == {64, 128, 256, 512, 1024, 2048}
    arr = np.array([t for t, _, _ in s])
    assert np.all(np.diff(arr) > 0)
    assert 0.5 * 400 / 200 < arr[-1] < 2.0 * 400 / 200  # mean rate 200/s
    sw = np.array([x for _, _, x in s]) / 1e-4
    assert sw.min() >= 1e3 * 0.999 and sw.max() <= 1e5 * 1.001
    for _, kw, _ in s:
        w = kw["sho_omega"][0]
        assert 0.5 <= w <= 2.0 and kw["node_temperature"] == w / 4.0


def test_admission_by_budget_and_completion():
    reqs = make_requests(60)
    budget = 3 * max(r.path.nbytes for r in reqs)
    fake = FakeServer(slots=8, budget=budget)
    loop = serving.ServeLoop(fake, round_budget=serving.DEFAULT_ROUND_BUDGET / 64)
    loop.run(reqs, realtime=False)
    assert fake.used == 0 and not fake.live
    assert fake.max_used <= budget and fake.max_live <= 8
    assert fake.max_live >= 2 and loop.overlapped > 0  # requests overlapped
    for r in reqs:
        ra = r.round_attempts
        assert 1 <= ra <= r.attempts
        assert r.done >= r.attempts and r.done - r.attempts < ra
        assert len(r.energies) == loop.samples_for(r) >= 1
        assert r.finished >= r.admitted >= r.arrival


def test_round_attempts_follow_cost():
    # a round costs about the same for every system: small systems take more attempts
    loop = serving.ServeLoop(FakeServer(1, 1))
    small = serving.Request(0, W.serve_stream(1)[0][1], [], None, 10 ** 6)
    small.system_kw = dict(small.system_kw, counts=[1, 1], nlevel=4)
    big = serving.Request(1, dict(small.system_kw, counts=[32, 32], nlevel=5), [], None, 10 ** 6)
    assert loop.round_attempts(big) == 8
    assert loop.round_attempts(small) > 100 * loop.round_attempts(big)


def test_same_samples_alone_and_in_mix():
    reqs = make_requests(20)
    budget = serving.DEFAULT_ROUND_BUDGET / 64
    loop = serving.ServeLoop(FakeServer(6, 1 << 40), round_budget=budget)
    loop.run(reqs, realtime=False)
    for k in (0, 7, 19):
        alone = make_requests(20)[k]
        serving.ServeLoop(FakeServer(6, 1 << 40), round_budget=budget).run([alone],
                                                                          realtime=False)
        assert alone.energies == reqs[k].energies


def test_never_admissible_raises():
    r = make_requests(1)[0]
    with pytest.raises(RuntimeError):
        serving.ServeLoop(FakeServer(2, 8)).run([r], realtime=False)


def test_summary_percentiles():
    reqs = make_requests(10)
    for i, r in enumerate(reqs):
        r.arrival, r.finished, r.done = 0.0, float(i + 1), 32
    s = serving.summary(reqs, wall=10.0)
    assert s["p50_s"] == pytest.approx(5.5) and s["p99_s"] == pytest.approx(9.91)
    assert s["bead_updates"] == sum(32 * ((1 << r.system_kw["nlevel"]) - 1) for r in reqs)
