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
    p.add_argument("--workload", default="dot20_fn", choices=["dot20_fn", "dot2", "heg54"])
    p.add_argument("--replicas", type=int, default=0, help="replicas per GPU (0: auto)")
    p.add_argument("--attempts", type=int, default=0, help="attempts per replica per step")
    p.add_argument("--precision", default="fp64", choices=["fp64", "mixed"])
    p.add_argument("--cpu-seconds", type=float, default=12.0)
    p.add_argument("--no-cpu-baseline", action="store_true")
    return p.parse_args()


def workload_kw(name):
    return {"dot20_fn": WL.dot20_fn, "dot2": WL.dot2, "heg54": WL.heg54}[name]()


def init_kind(name):
    return {"dot20_fn": "const", "dot2": "gauss", "heg54": "grid"}[name]


def defaults(name):
    # replicas per GPU and attempts per replica per step (0: one sweep)
    return {"dot20_fn": (608, 0), "dot2": (9728, 0), "heg54": (152, 1)}[name]


def sweep_attempts(kw):
    """Section attempts in one sweep: ceil(M / 2^L) sections times N particles."""
    L = kw["nlevel"]
    return -(-kw["nslice"] // (1 << L)) * sum(kw["counts"])


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
def _cpu_worker(args):
    kw, seed, replica, seconds = args
    # pi-qmc's constructors print progress to stdout; keep the JSON line clean
    devnull = os.open(os.devnull, os.O_WRONLY)
    os.dup2(devnull, 1)
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    sys.path.insert(0, os.path.join(REPO, "pi-qmc_gb300"))
    import oracle_lib as O
    import pimc_gb300
    tabs, ew = pimc_gb300.coulomb_tables(kw)
    cfg = O.make_config(**dict(kw, seed=seed, replica=replica))
    if O.RefOracle.available():
        sim = O.RefOracle(cfg)
    else:
        sim = O.PortOracle(cfg, tabs, ew)
    sim.set_path(WL.initial_path(cfg, init_kind_for(kw), seed=seed + replica))
    # pi-qmc's loop body: a sweep of section moves, then one energy measurement
    chunk = sweep_attempts(kw)
    n, t0 = 0, time.perf_counter()
    while time.perf_counter() - t0 < seconds:
        sim.run(chunk, first_attempt=n)
        sim.thermo_energy()
        n += chunk
    dt = time.perf_counter() - t0
    return n, dt


def init_kind_for(kw):
    if kw.get("ewald"):
        return "grid"
    return "const" if any(kw.get("node_kind", [0])) else "gauss"


def cpu_throughput(kw, seconds, cores):
    """Bead-updates/s of the CPU implementation on `cores` processes."""
    ctx = mp.get_context("spawn")
    L = kw["nlevel"]
    with ctx.Pool(cores) as pool:
        res = pool.map(_cpu_worker, [(kw, 777, r, seconds) for r in range(cores)])
    attempts = sum(n for n, _ in res)
    wall = max(dt for _, dt in res)
    return attempts * ((1 << L) - 1) / wall, attempts


def cpu_kind():
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle_lib as O
    return "reference" if O.RefOracle.available() else "port"


# ---------------------------------------------------------------- engine arm
def run_engine(args, rank, world):
    import torch
    import pimc_gb300

    torch.cuda.set_device(0 if world == 1 else int(os.environ.get("LOCAL_RANK", rank)))
    kw = workload_kw(args.workload)
    R0, A0 = defaults(args.workload)
    R = args.replicas or R0
    A = args.attempts or A0 or sweep_attempts(kw)
    L = kw["nlevel"]
    prec = pimc_gb300.PIMC_PREC_MIXED if args.precision == "mixed" else pimc_gb300.PIMC_PREC_FP64
    tabs, ew = pimc_gb300.coulomb_tables(kw)
    eng = pimc_gb300.Engine(kw, R, tabs, ew, seed=20261203 + 1000003 * rank, precision=prec)
    stream = torch.cuda.current_stream()
    eng.set_stream(stream.cuda_stream)
    cfg_shape = (kw["nslice"], sum(kw["counts"]), 3)

    class _C:
        nslice, npart, cell = kw["nslice"], sum(kw["counts"]), [kw.get("cell", 1000.0)] * 3

    paths = np.concatenate([WL.initial_path(_C, init_kind(args.workload), seed=100 + r).ravel()
                            for r in range(R)])
    host = torch.from_numpy(paths).pin_memory()
    eng.upload_paths(paths)
    # depth statistics for the flop model (untimed)
    rec = eng.run_sections(4, records=True)
    rl = rec["reject_level"].ravel()
    reach = [float(np.mean((rl < 0) | (rl <= lev))) for lev in range(L + 1)]
    eng.upload_paths(paths)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    for _ in range(args.warmup):
        eng.run_sections(A)
        energy = eng.thermo_energy()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    n_launch0 = eng.kernel_launches
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    with ClockSampler() as clk:
        torch.cuda.synchronize()
        for i in range(args.steps):
            flush.fill_(float(i))
            ev[i][0].record(stream)
            eng.run_sections(A)
            energy = eng.thermo_energy()
            ev[i][1].record(stream)
        torch.cuda.synchronize()
    launches = eng.kernel_launches - n_launch0
    step_ms = [a.elapsed_time(b) for a, b in ev]
    t_ms = sum(step_ms)
    if world > 1:
        t = torch.tensor([t_ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        t_ms = float(t.item())
    units = R * A * ((1 << L) - 1)
    value = world * units * args.steps / (t_ms * 1e-3)
    # ---- end to end through the public API, host buffers each step
    e2e_steps = max(2, min(args.steps, 5))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        eng.upload_paths(host.numpy())
        eng.run_sections(A)
        energy = eng.thermo_energy()
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    e2e_value = world * units * e2e_steps / e2e_s
    # ---- roofline of the dominant kernel (the section-move kernel)
    fp64_peak = pimc_gb300.fp64_peak_tflops()
    flops = attempt_flops(kw, reach) * R * A
    achieved = flops / (t_ms / args.steps * 1e-3) / 1e12
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if args.precision == "fp64" else "f32+f64",
        "data": "synthetic (seeded initial paths; Philox4x32-10 proposals)",
        "config": {"workload": f"{args.workload}: " + describe(args.workload),
                   "step": "one sweep of section moves per replica + one thermodynamic "
                           "energy measurement per replica",
                   "replicas_per_gpu": R, "attempts_per_replica_per_step": A,
                   "bead_updates_per_attempt": (1 << L) - 1, "precision": args.precision,
                   "l2": "paths (%.0f MB) exceed L2 and a 256 MB buffer is written between steps"
                         % (paths.nbytes / 1e6),
                   "parallelism": f"replicas{world}"},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(paths.nbytes),
                "d2h_bytes_per_step": int(R * 8),
                "path": "pimc_upload_paths (pinned host) + pimc_run_sections + pimc_thermo_energy"},
        "gpu_launches": int(launches),
        "roofline": {"bound": "fp64", "achieved": achieved, "peak": fp64_peak,
                     "unit": "TFLOP/s", "frac": achieved / fp64_peak,
                     "peak_source": "measured FP64 FMA probe (pimc_fp64_peak); "
                                    "MEASURED_PEAKS.json holds no FP64 figure",
                     "traffic": None, "kernel": "section_moves_kernel",
                     "flops_per_attempt_model": attempt_flops(kw, reach),
                     "level_reach": reach},
        "clocks": clk.summary(),
        "energy_mean": float(np.mean(energy)),
    }
    return out


def describe(name):
    return {
        "dot20_fn": "3-D harmonic dot, N=20 (10 up, 10 down), SHONodes fixed node, beta=20, "
                    "M=1024, level 5, Coulomb pair action norder 3",
        "dot2": "3-D harmonic dot, N=2 (1 up, 1 down), beta=10, M=256, level 4, Coulomb "
                "pair action norder 3",
        "heg54": "electron gas, N=54, r_s=4, T/T_F=0.5, Ewald |k|<5(2pi/L), "
                 "FreeParticleNodes 27x27, M=512, level 5",
    }[name]


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if args.impl == "engine" else "gloo")
    if args.impl == "reference":
        if rank == 0:
            kw = workload_kw(args.workload)
            cores = os.cpu_count() or 1
            t0 = time.perf_counter()
            value, attempts = cpu_throughput(kw, max(2.0, args.cpu_seconds / 2), cores)
            wall = time.perf_counter() - t0
            kind = cpu_kind()
            out = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
                   "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
                   "ms_per_step": wall * 1e3, "higher_is_better": True, "scaling": "weak",
                   "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                   "config": {"workload": f"{args.workload}: " + describe(args.workload)},
                   "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": kind,
                                    "sample": f"{attempts} section attempts over {cores} "
                                              f"processes, one replica each"},
                   "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}}
            print(json.dumps(out))
        return
    out = run_engine(args, rank, world)
    if rank == 0:
        if not args.no_cpu_baseline:
            kw = workload_kw(args.workload)
            cores = os.cpu_count() or 1
            v, att = cpu_throughput(kw, args.cpu_seconds, cores)
            out["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": cores, "kind": cpu_kind(),
                                   "sample": f"{att} section attempts of the same workload "
                                             f"over {cores} processes ({args.cpu_seconds:.0f} s)"}
        print(json.dumps(out))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
