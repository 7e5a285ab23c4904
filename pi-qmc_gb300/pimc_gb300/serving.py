"""Serving loop: continuous batching of simulations on one GPU.

Requests (a system, its pair tables, an initial path and a number of section
attempts) arrive over time.  The loop admits each arrived request into a free
slot of a :class:`pimc_gb300.Server` as soon as a slot and device memory for its
path and Slater-result cache are free (first fit over the waiting requests in
arrival order), then runs one round: every admitted simulation advances its own
number of section attempts in one persistent launch, then the thermodynamic
energy is measured for the slots that completed a sweep (ceil(M / 2^L) N
attempts, pi-qmc's measurement interval) or their whole request in that
round.  Simulations that have done their attempts
leave and free their slots for the next arrivals.  Work of requests that
arrive while others run overlaps on the device.

A round should take about the same device time for every slot, so a slot's
attempts per round are the round's cost budget divided by the cost of one of
its attempts (:func:`attempt_cost`, from its own system only).  A simulation
draws the random stream of its request id, so its chain, its rounds and its
energy samples do not depend on which other requests share the device.

This is the device-resident counterpart of running pi-qmc's
``<Loop><ChooseSection/><Sample/><Measure/></Loop>`` (src/parser/PIMCParser.cc)
once per simulation: each round is one ``ChooseSection``/``Sample`` block per
slot followed by ``ThermoEnergyEstimator`` (src/estimator/ThermoEnergyEstimator.cc).
"""
import collections
import math
import time
from dataclasses import dataclass, field

import numpy as np


@dataclass
class Request:
    rid: int
    system_kw: dict
    tables: list
    path: np.ndarray
    attempts: int
    arrival: float = 0.0
    # filled by the loop
    slot: int = -1
    admitted: float = math.nan
    finished: float = math.nan
    done: int = 0
    energies: list = field(default_factory=list)
    final_path: np.ndarray = None

    round_attempts: int = 0

    @property
    def beads(self):
        """Bead updates the request asked for: attempts x (2^L - 1)."""
        return self.attempts * ((1 << self.system_kw["nlevel"]) - 1)

    @property
    def latency(self):
        return self.finished - self.arrival

    def result(self, discard=0.2):
        """Mean thermodynamic energy after discarding the first `discard`
        fraction of samples, and its standard error from blocks of samples."""
        e = np.asarray(self.energies, float)
        e = e[int(len(e) * discard):] if len(e) > 1 else e
        if len(e) == 0:
            return math.nan, math.nan
        nb = min(16, len(e))
        blocks = np.array([b.mean() for b in np.array_split(e, nb)])
        err = blocks.std(ddof=1) / math.sqrt(nb) if nb > 1 else math.nan
        return float(e.mean()), float(err)


def attempt_cost(kw):
    """Relative device time of one section attempt of a system: pair terms
    over the links of every level (N^2 2^L) plus, per node species of n
    particles, Slater evaluations of the moved slices (n^2 (n + 20) 2^L)."""
    n_all = sum(kw["counts"])
    links = 1 << kw["nlevel"]
    c = float(n_all * n_all)
    for i, n in enumerate(kw["counts"]):
        if kw.get("node_kind", [0] * len(kw["counts"]))[i]:
            c += 2.0 * n * n * (n + 20)
    return c * links


# cost of 8 attempts of the largest served system (N=64, 32 per spin, level 5)
DEFAULT_ROUND_BUDGET = 8 * attempt_cost(dict(counts=[32, 32], nlevel=5, node_kind=[1, 1]))


class ServeLoop:
    """Drives a Server (or any object with admit/release/run/energies/
    download_path) over a list of requests."""

    def __init__(self, server, round_budget=DEFAULT_ROUND_BUDGET, max_round_attempts=4096,
                 keep_paths=False, clock=time.perf_counter):
        self.server = server
        self.budget = float(round_budget)
        self.max_ra = int(max_round_attempts)
        self.keep_paths = keep_paths
        self.clock = clock
        self.rounds = 0
        self.busy = 0.0
        self.overlapped = 0  # admissions while other simulations were running

    def round_attempts(self, req):
        if not req.round_attempts:
            ra = int(self.budget // attempt_cost(req.system_kw))
            req.round_attempts = max(1, min(self.max_ra, ra, req.attempts))
        return req.round_attempts

    def rounds_for(self, req):
        ra = self.round_attempts(req)
        return max(1, -(-req.attempts // ra))

    @staticmethod
    def sweep(req):
        """Section attempts of one sweep: ceil(M / 2^L) sections x N particles."""
        kw = req.system_kw
        return -(-kw["nslice"] // (1 << kw["nlevel"])) * sum(kw["counts"])

    def samples_for(self, req):
        """Energy samples a request gets: one per completed sweep, and one at its end."""
        ra, sw = self.round_attempts(req), self.sweep(req)
        n, done = 0, 0
        for _ in range(self.rounds_for(req)):
            prev, done = done, done + ra
            if done >= req.attempts or done // sw > prev // sw:
                n += 1
        return n

    def run(self, requests, realtime=True):
        """Serves `requests` (sorted by arrival).  With `realtime`, a request
        is admitted no earlier than its arrival time after the start; without,
        all are waiting at the start.  Returns the requests, filled in."""
        pending = collections.deque(sorted(requests, key=lambda r: r.arrival))
        waiting = []
        active = {}
        t0 = self.clock()
        now = lambda: self.clock() - t0  # noqa: E731
        if not realtime:
            for r in pending:
                r.arrival = 0.0
        while pending or waiting or active:
            t = now()
            while pending and pending[0].arrival <= t:
                waiting.append(pending.popleft())
            still = []
            for r in waiting:
                slot = self.server.admit(r.system_kw, r.tables, r.path, r.rid,
                                         self.round_attempts(r))
                if slot is None:
                    still.append(r)
                    continue
                r.slot = slot
                r.admitted = now()
                if active:
                    self.overlapped += 1
                active[slot] = r
            waiting = still
            if not active:
                if pending:
                    time.sleep(max(0.0, min(0.01, pending[0].arrival - now())))
                elif waiting:
                    raise RuntimeError(f"request {waiting[0].rid} can never be admitted")
                continue
            tb = self.clock()
            self.server.run()
            due = []
            for slot, r in active.items():
                prev = r.done
                r.done += r.round_attempts
                sw = self.sweep(r)
                if r.done >= r.attempts or r.done // sw > prev // sw:
                    due.append(slot)
            e = self.server.energies(due)
            self.busy += self.clock() - tb
            self.rounds += 1
            for k, slot in enumerate(due):
                active[slot].energies.append(float(e[k]))
            for slot in list(active):
                r = active[slot]
                if r.done >= r.attempts:
                    if self.keep_paths:
                        r.final_path = self.server.download_path(slot)
                    self.server.release(slot)
                    r.finished = now()
                    del active[slot]
        return requests


def summary(requests, wall):
    """p50/p99 time-to-result and aggregate bead-updates/s of a served stream."""
    lat = np.array([r.latency for r in requests])
    beads = sum(r.done * ((1 << r.system_kw["nlevel"]) - 1) for r in requests)
    return {
        "requests": len(requests),
        "p50_s": float(np.percentile(lat, 50)),
        "p99_s": float(np.percentile(lat, 99)),
        "mean_s": float(lat.mean()),
        "bead_updates": int(beads),
        "wall_s": wall,
        "bead_updates_per_s": beads / wall if wall > 0 else math.nan,
    }
