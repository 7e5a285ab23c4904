"""Throughput benchmark of the bisection hot path: attempted bead-updates/s.

Workload (default): the fixed-node harmonic dot — 20 electrons (10 up, 10
down), SHONodes free-oscillator nodes (two 10x10 Slater determinants per
slice), beta=20, M=1024 slices, bisection level 5, Coulomb pair action
(norder 3), omega=1 — run as R independent replicas (clones) of that system on
one GPU.  One step = the body of pi-qmc's main loop: one sweep of section-move
attempts on every replica (ceil(M/2^L) * N = 640 attempts; `--attempts`
overrides) followed by one thermodynamic-energy measurement of every replica.
One attempted bead-update = one interior bead proposed by a bisection move,
nmoving*(2^L-1) = 31 per attempt, counted whether or not a level rejects.

Data: synthetic (seeded constant-in-time initial paths, one N(0,1) point per
particle); no dataset.  Inputs (all replicas' paths, ~0.6 GB) are larger than
L2, and L2 is also flushed between timed steps.

--impl reference runs the reference's CPU implementation of the same
workload on all host cores (the C++ restatement of pi-qmc's code when the
reference build is not present on the machine).
"""
import argparse
import hashlib
import json
import math
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(REPO, "pi-qmc_gb300"))

import numpy as np  # noqa: E402

from pimc_gb300 import workloads as WL  # noqa: E402

METRIC = "bead-updates/s on 1 GB300 (batched vs plain, same E error); p50/p99 latency"
UNIT = "bead-updates/s"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="engine", choices=["engine", "reference"])
    p.add_argument("--workload", default="dot20_fn",
                   choices=["dot20_fn", "dot2", "heg54", "batch4096", "serve"])
    p.add_argument("--replicas", type=int, default=0, help="replicas per GPU (0: auto)")
    p.add_argument("--attempts", type=int, default=0, help="attempts per replica per step")
    p.add_argument("--precision", default="auto", choices=["auto", "fp64", "mixed"],
                   help="auto: the precision the workload is specified in (FP64 for dot2, "
                        "FP32 bulk + FP64 determinants for the others)")
    p.add_argument("--cpu-seconds", type=float, default=12.0,
                   help="timed seconds of the engine line's all-core CPU baseline")
    p.add_argument("--equil", type=int, default=-1,
                   help="untimed equilibration rounds before the warm-up (-1: per workload)")
    p.add_argument("--serve-requests", type=int, default=600,
                   help="requests of the serving sub-run in the default line (0: none)")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--other-configs", default="dot2,heg54,batch4096",
                   help="workloads measured in short sub-runs of the default line ('' : none)")
    p.add_argument("--no-autotune", action="store_true", help="keep the default launch shape")
    p.add_argument("--launch", default="",
                   help="block,scratch_global,regs_variant: this launch shape, no autotuning")
    p.add_argument("--requests", type=int, default=2000, help="serve: requests in the stream")
    p.add_argument("--rate", type=float, default=200.0, help="serve: mean arrivals per second")
    p.add_argument("--sweep-scale", type=float, default=1e-5,
                   help="serve: factor on the requested sweeps (log-uniform 1e3..1e5)")
    p.add_argument("--slots", type=int, default=1024, help="serve: concurrent simulations")
    p.add_argument("--server-block", type=int, default=256, help="serve: threads per simulation")
    p.add_argument("--server-scratch", type=int, default=0,
                   help="serve: Slater scratch placement (0 shared, 1 global, 2 split)")
    p.add_argument("--pool-gb", type=float, default=32.0, help="serve: device pool for paths")
    p.add_argument("--round-budget", type=float, default=1.0,
                   help="serve: round length in units of 8 attempts of the largest system")
    return p.parse_args()


def workload_kw(name):
    if name == "serve":
        return [kw for _, kw, _ in WL.serve_stream(64)]
    if name == "batch4096":
        return WL.batch_dots(4096)
    return {"dot20_fn": WL.dot20_fn, "dot2": WL.dot2, "heg54": WL.heg54}[name]()


def init_kind(name):
    return {"dot20_fn": "const", "dot2": "gauss", "heg54": "grid", "batch4096": "const",
            "serve": "const"}[name]


def defaults(name):
    # replicas per GPU and attempts per replica per step (0: one sweep)
    return {"dot20_fn": (608, 0), "dot2": (9728, 0), "heg54": (152, 64),
            "batch4096": (4096, 32), "serve": (64, 64)}[name]


def workload_precision(name, requested):
    if requested != "auto":
        return requested
    return "fp64" if name == "dot2" else "mixed"


def sweep_attempts(kw):
    """Section attempts in one sweep: ceil(M / 2^L) sections times N particles."""
    L = kw["nlevel"]
    return -(-kw["nslice"] // (1 << L)) * sum(kw["counts"])


# ------------------------------------------------------- measured work per unit
# Thread-level FP64 flops (DADD + DMUL + 2 DFMA), FP32 flops (FADD + FMUL +
# 2 FFMA), predicated-on lanes only, and DRAM bytes (read + write) per section
# attempt of the section kernel, counted by ncu on the same kernel and workload
# after a warm-up step.  `sha` is kernel_source_sha() of the build they were
# counted on: another build's counts are not used (the line then falls back to
# the operation-count model and says so).
MEASURED_WORK = {
    # launch shape of the count (block, scratch placement, register variant):
    # the DRAM bytes depend on the scratch placement, the flops do not
    ("dot20_fn", "mixed"): dict(fp64=3.220e5, fp32=1.895e5, dram=1.082e5, shape="256,0,2",
                                sha="6f18248147df49dd"),
    ("dot20_fn", "fp64"): dict(fp64=6.504e5, fp32=4.475e3, dram=1.141e5, shape="256,2,2",
                               sha="6f18248147df49dd"),
    # counted on the first 1024 replicas of the mix
    ("batch4096", "mixed"): dict(fp64=1.474e5, fp32=8.393e4, dram=3.358e4, shape="128,2,2",
                                 sha="6f18248147df49dd"),
    ("heg54", "mixed"): dict(fp64=1.891e6, fp32=5.344e5, dram=3.924e6, shape="512,1,1",
                             sha="6f18248147df49dd"),
    ("dot2", "fp64"): dict(fp64=1.760e4, fp32=164.4, dram=558.3, shape="32,0,3",
                           sha="6f18248147df49dd"),
}


# ---------------------------------------------------------------- flop model
def attempt_flops(kw, reach):
    """Algorithmic FP64 work of one section-move attempt (flops; an FMA is 2,
    exp/log 20, sqrt and division 8), weighted by reach[l] = the fraction of
    attempts that evaluate level l.  Counted from the kernel's loops:
    links 2^(L-l) per level (new and old path each), partners N-1 per link,
    moved slices 2^(L-l-1) with two Box-Muller pairs each, Slater matrices
    n x n per changed slice (build n^2 exp, LU 2/3 n^3, inverse 4/3 n^3,
    distances 2 n^2 (exp + 20)), and the set-up evaluation of every section
    slice for both node species (LU only for the species that does not move)."""
    L = kw["nlevel"]
    N = sum(kw["counts"])
    TR, SQ = 20.0, 8.0
    fixed = any(kw.get("node_kind", [0]))
    ns = max(kw["counts"]) if fixed else 0
    nsec = (1 << L) + 1
    total = 0.0
    for lev in range(L, -1, -1):
        links = 1 << (L - lev)
        nmov = 0 if lev == L else 1 << (L - lev - 1)
        f = 0.0
        f += nmov * (2 * (2 * TR + 2 * SQ + 60) + 40)          # mover
        f += links * 2 * (12 + 18)                             # spring + SHO
        if kw.get("coulomb"):
            f += links * 2 * (N - 1) * (45 + 2 * SQ + TR + 8)  # pair action
        if fixed:
            nchg = 1 if lev == L else 1 << (L - lev - 1)
            full = ns * ns * (TR + 8) + (2.0 / 3 + 4.0 / 3) * ns ** 3 * 2 + 2 * ns * ns * (TR + 20)
            f += nchg * full
            if lev == 0:
                f += (nsec - 1) * ns * 2 * (2 * TR + 6)        # nodal action
        total += reach[lev] * f
    if fixed:
        full = ns * ns * (TR + 8) + 2.0 * ns ** 3 * 2 + 2 * ns * ns * (TR + 20)
        lu = ns * ns * (TR + 8) + (2.0 / 3) * ns ** 3 * 2
        total += nsec * (full + lu)
    return total


# ----------------------------------------------------------- ranks (torchrun)
def max_over_ranks(x, world, device="cuda"):
    """The largest x over the ranks (the job's time is its slowest rank's)."""
    if world <= 1:
        return float(x)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def rank_seed(rank):
    """Each rank runs its own replicas: distinct random streams per rank."""
    return 20261203 + 1000003 * rank


# ---------------------------------------------------------------- clocks
class ClockSampler:
    def __init__(self):
        self.rows = []
        self.proc = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL,
                                         text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(2)
            except Exception:
                self.proc.kill()

    def summary(self, device=0):
        rows = [r for r in self.rows if len(r) >= 9 and r[0] == str(device)]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(rows)}


# ---------------------------------------------------------------- CPU side
# The CPU implementation of the path: pi-qmc's own hot-path code (oracle/_ref)
# where the reference tree was built on this machine, else the C++
# restatement (oracle/liboracle_port.so).  It loads nothing from the engine:
# pi-qmc builds its own tables, and the restatement takes the tables pi-qmc
# built for these workloads from the golden fixtures.
def reference_tables(kw):
    """pi-qmc's pair tables (and Ewald table) for a bench workload's system."""
    sys.path.insert(0, os.path.join(REPO, "tests"))
    import golden_io
    import workloads as TW
    for name, (gkw, _, _) in TW.GOLDEN_CASES.items():
        if gkw == kw:
            g = golden_io.load(name)
            return g["tables"], g["ewald"]
    mix = golden_io.load_tables("dot_mix")
    base = mix["kw"]
    same = all(kw.get(k, 1.0) == base.get(k, 1.0) for k in ("masses", "charges", "cell"))
    if same and abs(kw["beta"] / kw["nslice"] - base["beta"] / base["nslice"]) < 1e-15:
        return WL.tables_for(kw, mix["tables"]), None
    raise KeyError("no pi-qmc tables recorded for this system")


def _cpu_worker(args):
    kw, seed, replica, warmup, steps, chunk = args
    # pi-qmc's constructors print progress to stdout; keep the JSON line clean
    devnull = os.open(os.devnull, os.O_WRONLY)
    os.dup2(devnull, 1)
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle_lib as O
    cfg = O.make_config(**dict(kw, seed=seed, replica=replica))
    if O.RefOracle.available():
        sim = O.RefOracle(cfg)
    else:
        tabs, ew = reference_tables(kw)
        sim = O.PortOracle(cfg, tabs, ew)
    sim.set_path(WL.initial_path(cfg, init_kind_for(kw), seed=seed + replica))
    # pi-qmc's loop body: `chunk` section attempts, then one energy measurement
    n = 0
    for _ in range(warmup):
        sim.run(chunk, first_attempt=n)
        sim.thermo_energy()
        n += chunk
    t0 = time.perf_counter()
    for _ in range(steps):
        sim.run(chunk, first_attempt=n)
        sim.thermo_energy()
        n += chunk
    dt = time.perf_counter() - t0
    return steps * chunk * ((1 << kw["nlevel"]) - 1), steps * chunk, dt


def init_kind_for(kw):
    if kw.get("ewald"):
        return "grid"
    return "const" if any(kw.get("node_kind", [0])) else "gauss"


def cpu_throughput(kws, steps, warmup, cores, chunk):
    """Bead-updates/s of the CPU implementation on `cores` processes: process p
    runs replica p of the workload through `warmup` untimed and `steps` timed
    steps of `chunk` attempts each.  Returns (value, attempts, timed wall of
    the slowest process)."""
    kws = kws if isinstance(kws, list) else [kws]
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores) as pool:
        res = pool.map(_cpu_worker, [(kws[r % len(kws)], 777, r, warmup, steps,
                                      chunk or sweep_attempts(kws[r % len(kws)]))
                                     for r in range(cores)])
    beads = sum(b for b, _, _ in res)
    wall = max(dt for _, _, dt in res)
    return beads / wall, sum(n for _, n, _ in res), wall


def cpu_kind():
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle_lib as O
    return "reference" if O.RefOracle.available() else "port"


def cpu_model():
    """The host CPU's model name (lscpu, else /proc/cpuinfo, else the machine)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    import platform
    return platform.machine()


def cpu_baseline(kws, chunk, seconds, cores):
    """The CPU implementation on all host cores, one process per replica stream,
    sized to about `seconds` of timed work, plus one process alone (the
    single-core rate).  Returns the cpu_baseline record."""
    one, _, w1 = cpu_throughput(kws, 1, 0, 1, chunk)  # one step alone: its length
    steps = max(1, int(round(seconds / max(w1, 1e-3))))
    single, _, _ = cpu_throughput(kws, max(1, steps // 2), 1, 1, chunk)
    value, attempts, wall = cpu_throughput(kws, steps, 1, cores, chunk)
    return {"value": value, "unit": UNIT, "cores": cores, "kind": cpu_kind(),
            "cpu_model": cpu_model(), "single_core_value": single,
            "all_core_per_core_value": value / cores,
            "sample": f"{cores} processes (one replica each, replicas 0..{cores - 1} of the "
                      f"workload), each 1 untimed and {steps} timed steps of "
                      f"{chunk or 'one sweep of'} section attempts + one energy "
                      f"measurement; {attempts} timed attempts in {wall:.1f} s"}


# ---------------------------------------------------------------- serving arm
def serve_requests(args, base, nreq, seed):
    from pimc_gb300 import serving
    out = []
    for i, (t, kw, sw) in enumerate(WL.serve_stream(nreq, rate=args.rate, seed=seed,
                                                    sweep_scale=args.sweep_scale)):
        att = max(1, int(round(sw * WL.sweep_attempts(kw))))
        path = WL.initial_path(kw, "const", seed=1000 + i) / math.sqrt(kw["sho_omega"][0])
        out.append(serving.Request(i, kw, WL.tables_for(kw, base), path, att, t))
    return out


def run_serve(args, rank, world):
    """Continuous batching of a Poisson stream of dot simulations: requests are
    admitted into server slots as slots and pool memory free up, every round
    advances each admitted simulation by its own attempts (sized so that a
    round costs about the same device time for every system) and measures their
    energies, and finished simulations leave.  value = bead
    updates of all requests / wall time from the first arrival to the last
    result; p50/p99 time-to-result per request."""
    import torch
    import pimc_gb300
    from pimc_gb300 import serving
    prec = pimc_gb300.PIMC_PREC_MIXED if args.precision == "mixed" else pimc_gb300.PIMC_PREC_FP64
    kw0 = WL.serve_stream(1)[0][1]
    base, _ = pimc_gb300.coulomb_tables(dict(kw0, counts=[2, 2], node_kind=[1, 1],
                                             node_omega=[1.0, 1.0], sho_omega=[1.0, 1.0]))
    seed = rank_seed(rank)
    pool = int(args.pool_gb * (1 << 30))
    srv = pimc_gb300.Server(args.slots, pool, 64, 2048, 5, 32, seed=seed, precision=prec)
    srv.configure(args.server_block, args.server_scratch, 2)
    stream = torch.cuda.current_stream()
    srv.set_stream(stream.cuda_stream)
    # warm-up: a short stream served all at once (untimed)
    warm = serve_requests(args, base, max(8, args.warmup * 8), seed=99)
    budget = args.round_budget * serving.DEFAULT_ROUND_BUDGET
    serving.ServeLoop(srv, round_budget=budget).run(warm, realtime=False)
    reqs = serve_requests(args, base, args.requests, seed=WL.DEFAULT_SEED + rank)
    loop = serving.ServeLoop(srv, round_budget=budget)
    n_launch0 = srv.kernel_launches()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    with ClockSampler() as clk:
        t0 = time.perf_counter()
        loop.run(reqs, realtime=True)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
    wall = max_over_ranks(wall, world)
    summ = serving.summary(reqs, wall)
    beads = summ["bead_updates"]
    offered = sum(r.beads for r in reqs) / max(reqs[-1].arrival, 1e-9)
    h2d = sum(r.path.nbytes for r in reqs)
    value = world * beads / wall
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": loop.rounds,
        "warmup": args.warmup, "ms_per_step": wall * 1e3 / max(1, loop.rounds),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if args.precision == "fp64" else "f32+f64",
        "data": "synthetic (seeded Poisson stream, seeded initial paths; Philox4x32-10 "
                "proposals)",
        "config": {"workload": "serve: " + describe("serve"),
                   "step": "one serving round: every admitted simulation advances its own "
                           "attempts (about equal device time each; 8 for N=64 at level 5), "
                           "then the simulations that completed a sweep or their request "
                           "are measured",
                   "requests": args.requests, "rate_per_s": args.rate,
                   "sweep_scale": args.sweep_scale, "slots": args.slots,
                   "server_block": args.server_block, "server_scratch": args.server_scratch,
                   "pool_bytes": pool, "precision": args.precision,
                   "offered_bead_updates_per_s": offered,
                   "l2": "request paths and Slater caches (GBs in total) exceed L2",
                   "parallelism": f"replicas{world}"},
        "latency": {"p50_s": summ["p50_s"], "p99_s": summ["p99_s"], "mean_s": summ["mean_s"],
                    "unit": "s, arrival to result"},
        "e2e": {"value": value, "unit": UNIT,
                "h2d_bytes_per_step": int(h2d / max(1, loop.rounds)),
                "d2h_bytes_per_step": int(args.slots * 8),
                "path": "pimc_server_admit (host path) + pimc_server_run + pimc_server_energy "
                        "per round + pimc_server_release"},
        "gpu_launches": int(srv.kernel_launches() - n_launch0),
        "gpu_busy_fraction": loop.busy / wall,
        "admitted_while_others_ran": loop.overlapped,
        "roofline": None,
        "clocks": clk.summary(),
    }
    return out


# ---------------------------------------------------------------- engine arm
def bench_config(args, R, A, batch, kw, path_bytes):
    """The `config` record, the same for both arms: the workload and one step."""
    L = kw["nlevel"]
    return {"workload": f"{args.workload}: " + describe(args.workload),
            "step": "one sweep of section moves per replica + one thermodynamic "
                    "energy measurement per replica",
            "replicas_per_gpu": R, "attempts_per_replica_per_step": A,
            "bead_updates_per_attempt": (1 << L) - 1 if not batch else "2^L-1 per replica",
            "precision": args.precision,
            "l2": "paths (%.0f MB) exceed L2 and a 256 MB buffer is written between steps"
                  % (path_bytes / 1e6),
            "parallelism": f"replicas{args.gpus}"}


def engine_setup(args):
    kws = workload_kw(args.workload)
    batch = isinstance(kws, list)
    if batch and args.replicas:
        kws = kws[:args.replicas]  # the first replicas of the mix (smaller profiling runs)
    R0, A0 = defaults(args.workload)
    R = len(kws) if batch else (args.replicas or R0)
    kw = kws[0] if batch else kws
    A = args.attempts or A0 or sweep_attempts(kw)
    return kws, batch, R, kw, A


def energy_stats(E, what):
    """Mean thermodynamic energy of measurements E [steps][replicas] and its
    standard error from the per-replica means (each replica an independent
    chain: one block per replica)."""
    E = np.asarray(E, float)
    per = E.mean(axis=0)
    ok = np.isfinite(per)
    v = per[ok]
    err = float(v.std(ddof=1) / math.sqrt(len(v))) if len(v) > 1 else None
    return {"value": float(v.mean()) if len(v) else None, "stat_err": err,
            "blocks": int(ok.sum()), "measurements": int(E.size),
            "unit": "Hartree (reduced units)", "when": what,
            "sigma": "standard error of the per-replica means (independent chains as blocks)"}


def run_engine(args, rank, world):
    import torch
    import pimc_gb300
    if args.workload == "serve":
        return run_serve(args, rank, world)

    torch.cuda.set_device(0 if world == 1 else int(os.environ.get("LOCAL_RANK", rank)))
    kws, batch, R, kw, A = engine_setup(args)
    prec = pimc_gb300.PIMC_PREC_MIXED if args.precision == "mixed" else pimc_gb300.PIMC_PREC_FP64
    seed = rank_seed(rank)
    if batch:
        base, _ = pimc_gb300.coulomb_tables(dict(kw, counts=[2, 2], node_kind=[1, 1],
                                                 node_omega=[1.0, 1.0], sho_omega=[1.0, 1.0]))
        eng = pimc_gb300.Engine.batch(kws, [WL.tables_for(k, base) for k in kws], seed=seed,
                                      precision=prec)
        systems = kws
    else:
        tabs, ew = pimc_gb300.coulomb_tables(kw)
        eng = pimc_gb300.Engine(kw, R, tabs, ew, seed=seed, precision=prec)
        systems = [kw] * R
    L = kw["nlevel"]
    stream = torch.cuda.current_stream()
    eng.set_stream(stream.cuda_stream)

    def shape_of(k):
        class _C:
            nslice, npart, cell = k["nslice"], sum(k["counts"]), [k.get("cell", 1000.0)] * 3
        return _C

    paths = np.concatenate([WL.initial_path(shape_of(systems[r]), init_kind(args.workload),
                                            seed=100 + r).ravel() for r in range(R)])
    eng.upload_paths(paths)
    # equilibration (untimed): the energy block below is taken on equilibrated chains
    rounds, ndisp, nsweep = default_equil(args.workload)
    if args.equil >= 0:
        rounds = args.equil
    for _ in range(rounds):
        if ndisp:
            eng.run_displace(ndisp, [1.0, 1.0, 1.0], 1, -1)
        eng.run_steps(A, nsweep, energies=False)
    equil = rounds * nsweep
    # launch configuration chosen by the autotuner on the equilibrated chains
    # (untimed; the chains are restored after every trial)
    if args.launch:
        b, g, v = (int(x) for x in args.launch.split(","))
        eng.configure(b, g, 0, v)
        tuned, tried = eng.launch_config(), []
    elif args.no_autotune:
        tuned, tried = eng.launch_config(), []
    else:
        tuned, tried = eng.autotune(min(A, 32))
    # depth statistics for the flop model (untimed; the chains continue)
    rec = eng.run_sections(4, records=True)
    Ls = np.array([k["nlevel"] for k in systems])[:, None]
    rl = rec["reject_level"]
    depth_reach = [float(np.mean((rl < 0) | (rl <= Ls - d))) for d in range(int(Ls.max()) + 1)]
    reach = [depth_reach[L - lev] for lev in range(L + 1)]
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    for _ in range(args.warmup):
        eng.run_steps(A, 1, energies=False)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    n_launch0 = eng.kernel_launches
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    E = np.empty((args.steps, R))
    with ClockSampler() as clk:
        torch.cuda.synchronize()
        for i in range(args.steps):
            flush.fill_(float(i))
            ev[i][0].record(stream)
            # one captured graph (sweep + measurement); the step's energies to the host
            E[i] = eng.run_steps(A, 1, energies=True)[0]
            ev[i][1].record(stream)
        torch.cuda.synchronize()
    launches = eng.kernel_launches - n_launch0
    step_ms = [a.elapsed_time(b) for a, b in ev]
    t_ms = max_over_ranks(sum(step_ms), world)
    units = A * sum((1 << k["nlevel"]) - 1 for k in systems)
    value = world * units * args.steps / (t_ms * 1e-3)
    energy_block = energy_stats(E, f"the {args.steps} timed steps, after {equil} equilibration "
                                   f"sweeps ({rounds * ndisp} rigid displacement attempts of one "
                                   f"particle's path, uniform in a 1 bohr box, among them) and "
                                   f"{args.warmup} warm-up steps from the initial paths")
    energy_block.update(energy_vs_reference(args.workload, energy_block, equil + args.warmup))
    # ---- end to end through the public API: each step uploads the chain's
    # current paths from pinned host memory, runs the sweep, measures, and
    # brings the energies and the paths back (the next step's input)
    e2e_steps = max(2, min(args.steps, 5))
    host = torch.empty(paths.size, dtype=torch.float64).pin_memory().numpy()
    eng.download_paths(out=host)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        eng.upload_paths(host)
        eng.run_sections(A)
        e2e_energy = eng.thermo_energy()
        eng.download_paths(out=host)
    torch.cuda.synchronize()
    e2e_s = max_over_ranks(time.perf_counter() - t0, world)
    e2e_value = world * units * e2e_steps / e2e_s
    assert np.all(np.isfinite(e2e_energy))
    # ---- the mixed form's error per result against the FP64 form (untimed)
    if args.precision == "mixed" and not batch:
        energy_block["precision_error"] = precision_report(pimc_gb300, kw, tabs, ew, paths, R, A,
                                                           seed, stream)
    # ---- the plain form: one replica, FP64, same sweep (untimed by the step loop)
    plain = None if batch else pimc_gb300.Engine(kw, 1, tabs, ew, seed=seed)
    plain_value = None
    if plain is not None:
        plain.set_stream(stream.cuda_stream)
        plain.upload_paths([paths[:3 * kw["nslice"] * sum(kw["counts"])]])
        plain.run_steps(A, 1, energies=False)
        a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a0.record(stream)
        plain.run_steps(A, 1, energies=False)
        a1.record(stream)
        torch.cuda.synchronize()
        plain_value = A * ((1 << L) - 1) / (a0.elapsed_time(a1) * 1e-3)
        plain.close()
    # ---- roofline of the dominant kernel (the section-move kernel), timed
    # alone with CUDA events on its stream over three more launches
    sec_ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(3)]
    torch.cuda.synchronize()
    for a0, a1 in sec_ev:
        flush.fill_(1.0)
        a0.record(stream)
        eng.run_sections(A)
        a1.record(stream)
    torch.cuda.synchronize()
    section_ms = statistics.mean(a0.elapsed_time(a1) for a0, a1 in sec_ev)
    roofline = section_roofline(args, systems, batch, kw, R, A, reach, depth_reach, section_ms,
                                pimc_gb300)
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if args.precision == "fp64" else "f32+f64",
        "data": "synthetic (seeded initial paths; Philox4x32-10 proposals)",
        "config": bench_config(args, R, A, batch, kw, paths.nbytes),
        "launch": {"chosen": tuned, "candidates": tried},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(paths.nbytes),
                "d2h_bytes_per_step": int(paths.nbytes + R * 8),
                "steps": e2e_steps,
                "path": "per step: pimc_upload_paths (the chain's current paths, pinned host) + "
                        "pimc_run_sections + pimc_thermo_energy + pimc_download_paths (pinned "
                        "host, the next step's input); the chain continues from the timed steps"},
        "gpu_launches": int(launches),
        "roofline": roofline,
        "clocks": clk.summary(),
        "energy": energy_block,
    }
    if plain_value is not None:
        out["plain_fp64_single_replica"] = {
            "value": plain_value, "unit": UNIT,
            "what": "the same step on one replica in FP64 (pimc_run_steps, CUDA events)"}
        out["batched_over_plain"] = value / plain_value
    return out


def precision_report(pimc_gb300, kw, tabs, ew, paths, R, A, seed, stream):
    """Error of every mixed-form result against the FP64 form on identical
    inputs.  Both forms draw the same FP64 proposals, so a mixed chain and an
    FP64 chain started from the same path and stream make the same moves until
    a decision differs (a uniform within the mixed error of its acceptance
    probability); on those common attempts each level's action difference,
    fixed-node difference and ln T are compared.  The thermodynamic estimator
    is compared on identical paths (the FP64 chain's final paths measured by
    both engines)."""
    nr = min(R, 152)
    n_att = min(A, 128)
    per = 3 * kw["nslice"] * sum(kw["counts"])
    sub = paths[:nr * per]
    L = kw["nlevel"]
    recs, engs = [], []
    for prec in (pimc_gb300.PIMC_PREC_MIXED, pimc_gb300.PIMC_PREC_FP64):
        e = pimc_gb300.Engine(kw, nr, tabs, ew, seed=seed, precision=prec)
        e.set_stream(stream.cuda_stream)
        e.upload_paths(sub)
        recs.append(e.run_sections(n_att, records=True))
        engs.append(e)
    m, f = recs
    same = np.ones(nr, bool)
    common = np.zeros((nr, n_att), bool)
    for a in range(n_att):
        ok = ((m["reject_level"][:, a] == f["reject_level"][:, a]) &
              (m["ipart"][:, a] == f["ipart"][:, a]) & (m["ifirst1"][:, a] == f["ifirst1"][:, a]))
        common[:, a] = same
        same &= ok
    out = {"replicas": nr, "attempts": n_att, "compared_attempts": int(common.sum()),
           "chains_identical_throughout": int(same.sum()), "per_level": []}
    for lev in range(L + 1):
        row = {"level": lev}
        for key in ("ds", "ds_node", "lnt"):
            a, b = m[key][:, :, lev], f[key][:, :, lev]
            # a level's values exist where the FP64 chain evaluated it
            ev = common & ((f["reject_level"] < 0) | (f["reject_level"] <= lev))
            d = np.abs(a - b)[ev & (np.abs(b) < 1e99)]
            row[key] = {"max": float(d.max()) if d.size else None,
                        "rms": float(np.sqrt(np.mean(d * d))) if d.size else None,
                        "n": int(d.size)}
        out["per_level"].append(row)
    fin = engs[1].download_paths(flat=True)
    engs[0].upload_paths(fin)
    e_m, e_f = engs[0].thermo_energy(), engs[1].thermo_energy()
    de = np.abs(e_m - e_f)
    out["thermo_energy"] = {"max": float(de.max()), "rms": float(np.sqrt(np.mean(de * de))),
                            "relative_max": float((de / np.abs(e_f)).max())}
    for e in engs:
        e.close()
    return out


def default_equil(name):
    """Untimed equilibration before the warm-up: (rounds, rigid-displacement
    attempts per replica per round, sweeps per round).  Bisection moves shift a
    path's centroid only slowly; from constant-in-time paths the config-2 dot's
    chains still spread ~175 Ha apart after 150 sweeps of bisection alone, while
    pi-qmc's DisplaceMoveSampler moves (whole-path shifts) bring them to a
    ~30 Ha spread and the mean from ~195 to ~146 Ha within 50 sweeps."""
    return {"dot20_fn": (10, 20, 5), "dot2": (40, 0, 5), "heg54": (0, 0, 1),
            "batch4096": (0, 0, 1), "serve": (0, 0, 1)}[name]


# equilibrated energies of pi-qmc's own code (tests/golden/make_energy.py) for
# the bench workloads that have one
REFERENCE_ENERGY = {"dot2": "dot2_full"}


def energy_vs_reference(name, block, equil_steps):
    """The bench's energy against pi-qmc's FP64 energy of the same system:
    |E - E_pi-qmc| <= 2 sqrt(sigma^2 + sigma_pi-qmc^2)."""
    case = REFERENCE_ENERGY.get(name)
    f = os.path.join(REPO, "tests", "golden", f"energy_{case}.npz") if case else None
    if not f or not os.path.exists(f):
        return {"reference": None}
    z = np.load(f)
    er, sr = float(z["energy"]), float(z["sigma"])
    sig = math.hypot(sr, block["stat_err"] or 0.0)
    d = block["value"] - er
    return {"reference": {"value": er, "stat_err": sr, "blocks": int(z["block_means"].size),
                          "what": f"pi-qmc's own code (FP64), {int(z['block_means'].shape[0])} "
                                  f"chains after {int(z['equil'])} sweeps, blocks of "
                                  f"{int(z['block'])} sweeps"},
            "diff_vs_reference": d, "diff_over_sigma": d / sig if sig else None,
            "within_2sigma_of_reference": bool(abs(d) <= 2 * sig),
            "relative_stat_err": (block["stat_err"] or 0.0) / abs(block["value"]),
            "equilibration_sweeps": equil_steps}


def kernel_source_sha():
    """Digest of the section kernel's sources: the counted work per attempt
    below belongs to the kernel these files build."""
    d = os.path.join(REPO, "pi-qmc_gb300", "csrc")
    h = hashlib.sha256()
    for f in ("section_kernel.cuh", "kernels.cuh", "pimc_device.cuh", "pimc_rng.h",
              "section_variants.cu"):
        h.update(f.encode())
        h.update(open(os.path.join(d, f), "rb").read())
    return h.hexdigest()[:16]


def section_roofline(args, systems, batch, kw, R, A, reach, depth_reach, section_ms, pimc_gb300):
    """FP64- and FP32-pipe rooflines of the section kernel: counted work per
    attempt x attempts per launch / the kernel's CUDA-event time, over the
    measured FMA peaks of this device."""
    fp64_peak = pimc_gb300.fp64_peak_tflops()
    fp32_peak = pimc_gb300.fp32_peak_tflops()
    work = MEASURED_WORK.get((args.workload, args.precision))
    sha = kernel_source_sha()
    stale = work is not None and work["sha"] != sha
    if work is not None and not stale:
        flops = work["fp64"] * R * A
        flops32 = work["fp32"] * R * A if work.get("fp32") is not None else None
        traffic = work["dram"] * R * A if work.get("dram") is not None else None
        source = ("ncu thread-level DADD+DMUL+2*DFMA (FP64) and FADD+FMUL+2*FFMA (FP32) per "
                  "attempt of this kernel build and workload x attempts per launch")
    else:
        if batch:
            flops = sum(attempt_flops(k, [depth_reach[k["nlevel"] - lev]
                                          for lev in range(k["nlevel"] + 1)])
                        for k in systems) * A
        else:
            flops = attempt_flops(kw, reach) * R * A
        flops32 = traffic = None
        source = ("operation-count model (attempt_flops): "
                  + ("the counted work belongs to another build of the kernel"
                     if stale else "no hardware count for this workload"))
    achieved = flops / (section_ms * 1e-3) / 1e12
    out = {"bound": "fp64", "achieved": achieved, "peak": fp64_peak, "unit": "TFLOP/s",
           "frac": achieved / fp64_peak, "traffic": traffic, "kernel": "section_moves_kernel",
           "section_ms_per_launch": section_ms, "flops_per_launch": flops,
           "flops_source": source, "count_stale": stale, "kernel_sha": sha,
           "count_launch_shape": work.get("shape") if work else None,
           "peak_source": "measured FP64 FMA probe (pimc_fp64_peak); MEASURED_PEAKS.json holds "
                          "no FP64 figure",
           "flops_per_attempt_model": attempt_flops(kw, reach), "level_reach": reach}
    if flops32 is not None:
        a32 = flops32 / (section_ms * 1e-3) / 1e12
        out["fp32"] = {"achieved": a32, "peak": fp32_peak, "unit": "TFLOP/s",
                       "frac": a32 / fp32_peak,
                       "peak_source": "measured FP32 FMA probe (pimc_fp32_peak)"}
    return out


# ---------------------------------------------------------------- other configs
def other_config_subrun(args, name):
    """A short run of another workload of the hot path (3 warm-up and 3 timed
    steps, its own equilibration and autotuned launch shape), reported
    compactly beside the headline: the same measurement as its own line."""
    sub = argparse.Namespace(**vars(args))
    sub.workload = name
    sub.precision = workload_precision(name, "auto")
    sub.steps, sub.warmup = 3, 3
    sub.replicas = sub.attempts = 0
    sub.equil = -1
    sub.launch = ""
    out = run_engine(sub, 0, 1)
    r = out["roofline"]
    e = out["energy"]
    keep = {"value": out["value"], "unit": out["unit"], "e2e": out["e2e"]["value"],
            "ms_per_step": out["ms_per_step"], "steps": sub.steps, "warmup": sub.warmup,
            "dtype": out["dtype"], "workload": out["config"]["workload"],
            "replicas": out["config"]["replicas_per_gpu"],
            "attempts_per_replica_per_step": out["config"]["attempts_per_replica_per_step"],
            "launch": out["launch"]["chosen"], "gpu_launches": out["gpu_launches"],
            "clocks": out["clocks"],
            "roofline": {k: r.get(k) for k in ("bound", "achieved", "peak", "unit", "frac",
                                              "traffic", "section_ms_per_launch",
                                              "count_stale")},
            "energy": {k: e.get(k) for k in ("value", "stat_err", "reference",
                                             "diff_over_sigma", "within_2sigma_of_reference")}}
    if "batched_over_plain" in out:
        keep["batched_over_plain"] = out["batched_over_plain"]
    return keep


# ---------------------------------------------------------------- serving sub-run
def serving_subrun(args):
    """A short run of the serving stream (config 5's distributions and arrival
    rate) carried in the default line: p50/p99 time-to-result."""
    sub = argparse.Namespace(**vars(args))
    sub.workload = "serve"
    sub.requests = args.serve_requests
    sub.warmup = 1
    sub.precision = "mixed"
    out = run_serve(sub, 0, 1)
    return {"value": out["value"], "unit": UNIT, "latency": out["latency"],
            "requests": sub.requests, "rate_per_s": sub.rate, "sweep_scale": sub.sweep_scale,
            "rounds": out["steps"], "wall_s": out["ms_per_step"] * out["steps"] / 1e3,
            "gpu_launches": out["gpu_launches"],
            "admitted_while_others_ran": out["admitted_while_others_ran"],
            "offered_bead_updates_per_s": out["config"]["offered_bead_updates_per_s"],
            "workload": describe("serve"),
            "scaling_note": SERVE_SCALING_NOTE}


SERVE_SCALING_NOTE = (
    "config 5 asks 1e3..1e5 sweeps per request; a request is one Markov chain whose section "
    "attempts depend on each other, and the largest (N=64, M=2048, 1e5 sweeps) is 4e8 "
    "dependent attempts, days of one chain on any device, so no stream of these requests "
    "completes in a bench run at any arrival rate.  The stream keeps config 5's arrival "
    "rate and size distributions and scales every request's sweeps by sweep_scale.")


def describe(name):
    return {
        "batch4096": "4096 harmonic-dot replicas, N uniform 2..32 (SHONodes per spin, node "
                     "temperature omega/4), omega uniform [0.5,2], M in {128,256,512,1024}, "
                     "beta=M/25.6, level 4 or 5, Coulomb pair action norder 3",
        "dot20_fn": "3-D harmonic dot, N=20 (10 up, 10 down), SHONodes fixed node, beta=20, "
                    "M=1024, level 5, Coulomb pair action norder 3",
        "serve": "Poisson stream of harmonic-dot simulations, N uniform 2..64 (SHONodes per "
                 "spin, node temperature omega/4), omega uniform [0.5,2], M uniform in "
                 "{64..2048} (powers of 2), beta=M/25.6, level 4 (M<=128) or 5, Coulomb pair "
                 "action norder 3, requested sweeps log-uniform 1e3..1e5 times sweep_scale",
        "dot2": "3-D harmonic dot, N=2 (1 up, 1 down), beta=10, M=256, level 4, Coulomb "
                "pair action norder 3",
        "heg54": "electron gas, N=54, r_s=4, T/T_F=0.5, Ewald |k|<5(2pi/L), "
                 "FreeParticleNodes 27x27, M=512, level 5",
    }[name]


def run_reference(args, world):
    """The reference arm: pi-qmc's CPU implementation of the same workload on
    all host cores (one process per replica stream; --steps timed steps after
    --warmup untimed ones, each the engine arm's step: A section attempts and
    one energy measurement per replica).  Loads no engine code."""
    kws, batch, R, kw, A = engine_setup(args)
    cores = os.cpu_count() or 1
    value, attempts, wall = cpu_throughput(kws, args.steps, args.warmup, cores, A)
    path_bytes = sum(3 * 8 * k["nslice"] * sum(k["counts"])
                     for k in (kws if batch else [kw] * R))
    return {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": wall * 1e3 / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded initial paths; Philox4x32-10 proposals)",
            "config": bench_config(args, R, A, batch, kw, path_bytes),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": cpu_kind(),
                             "cpu_model": cpu_model(), "all_core_per_core_value": value / cores,
                             "sample": f"{cores} processes, one replica each (replicas "
                                       f"0..{cores - 1} of the workload), each {args.warmup} "
                                       f"untimed and {args.steps} timed steps of {A} section "
                                       f"attempts + one energy measurement; {attempts} timed "
                                       f"attempts, slowest process {wall:.2f} s"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}


def main():
    args = parse()
    args.precision = workload_precision(args.workload, args.precision)
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    args.gpus = world
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if args.impl == "engine" else "gloo")
    if args.impl == "reference":
        if rank == 0:
            print(json.dumps(run_reference(args, world)))
        return
    out = run_engine(args, rank, world)
    if rank == 0 and world == 1:
        if args.workload != "serve" and args.serve_requests > 0:
            out["serving"] = serving_subrun(args)
        if args.workload == "dot20_fn" and args.other_configs:
            # configs 1, 3 and 4 of the hot path, each measured as its own line
            # would be (`--workload <name>`), in short form
            out["other_configs"] = {w: other_config_subrun(args, w)
                                    for w in args.other_configs.split(",") if w}
        if not args.no_cpu_baseline:
            kws, batch, R, kw, A = engine_setup(args)
            out["cpu_baseline"] = cpu_baseline(kws, A, args.cpu_seconds, os.cpu_count() or 1)
    if rank == 0:
        print(json.dumps(out))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
