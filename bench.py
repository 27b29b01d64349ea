#!/usr/bin/env python
"""Benchmark of the GB300 engine on Lumol's MD / MC hot path.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                    [--workload lj_batch|serving|nacl_ewald|argon|water] [--precision mixed|fp64]

Default workload (lj_batch): 256 seeded argon-type LJ replicas of uneven size
(64..4096 atoms), half running NVT Velocity-Verlet MD in one engine, half
running NVT Monte Carlo Translate chains in another; one batched step is one
Lumol step of every replica (an MD step of each MD replica, one move of each
chain), and `value` is atom-steps/s (MD atoms + MC chains per step) of the
whole job, timed with CUDA events on the engines' streams.  With the mixed
path (default) the line also carries the plain FP64 path's value on the same
workload (`fp64_plain`, with the ratio) and the mixed path's error against
FP64 (`accuracy`: relative force RMS, energy and virial errors, NVE drift of
both paths).

The single-system workloads (nacl_ewald, argon, water) time one lg_md_run
call of `--chunk` MD steps per iteration, with the L2 cache flushed (256 MiB
write) before every timed iteration because those workloads fit in L2.  The
serving workload replays a seeded Poisson stream of mixed MD requests through
the continuous-batching server and reports throughput and p50 / p99 latency.
`e2e` is the same metric through the public C ABI with the state copied from
pinned host memory and back every step.

`--impl reference` times the reference algorithm on the host cores: the CPU
oracle (a C++ restatement of lumol-core's O(N^2) loops, OpenMP over all
cores), on the same workload and metric.  With torchrun (N > 1) every rank
runs an independent replica (the path has no exchange between systems);
rank 0 prints the line.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "atom-steps/s"
L2_FLUSH_BYTES = 256 << 20


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=200)
    p.add_argument("--warmup", type=int, default=10)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--workload", default="lj_batch", choices=["lj_batch", "serving", "nacl_ewald", "argon", "water"])
    p.add_argument("--requests", type=int, default=48, help="serving: number of requests")
    p.add_argument("--rate", type=float, default=40.0, help="serving: Poisson arrival rate (1/s)")
    p.add_argument("--replicas", type=int, default=256, help="lj_batch: replicas (half MD, half MC)")
    p.add_argument("--precision", default="mixed", choices=["fp64", "mixed"])
    p.add_argument("--cells", type=int, default=0, help="lattice cells per side (0: the workload's size)")
    p.add_argument("--chunk", type=int, default=256,
                   help="MD steps per timed iteration (one lg_md_run call; one persistent launch up to 256)")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-roofline", action="store_true")
    p.add_argument("--no-accuracy", action="store_true", help="skip the mixed-vs-FP64 error report")
    p.add_argument("--no-fp64-leg", action="store_true", help="lj_batch: skip timing the plain FP64 path")
    p.add_argument("--threads-per-atom", type=int, default=0,
                   help="lj_batch: fixed pair-kernel group size of the MD engine (0: autotuned)")
    p.add_argument("--no-configs", action="store_true",
                   help="lj_batch: skip the single-system (argon, NaCl, water) and serving legs")
    return p.parse_args()


def make_system(name: str, precision: str, cells: int = 0):
    from lumol_gb300 import workloads
    if name == "nacl_ewald":
        c = cells or 5
        s = workloads.nacl_crystal(cells=c, precision=precision)
        return s, 1.0, (f"NaCl rock salt {c}x{c}x{c} ({s.size} ions, L={5.64 * c:.1f} A), LJ rc=9 A, "
                        "Ewald rc=9 A alpha=0.35 kmax=7, NVE Velocity-Verlet dt=1 fs")
    if name == "argon":
        c = cells or 5
        s = workloads.argon_fcc(cells=c, precision=precision)
        return s, 1.0, (f"Argon FCC {c}x{c}x{c} ({s.size} atoms, L={5.76 * c:.1f} A), shifted LJ rc=10 A, "
                        "NVE Velocity-Verlet dt=1 fs")
    c = cells or 12
    s = workloads.water_box(n_side=c, length=37.3 * c / 12, precision=precision)
    return s, 0.5, (f"SPC/E-geometry flexible water {c}^3 ({s.size} atoms, L={37.3 * c / 12:.1f} A), Ewald "
                    "alpha=0.3 kmax=8 rc=10 A, harmonic bonds/angles, Velocity-Verlet dt=0.5 fs")


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(world, value: float) -> float:
    if world == 1:
        return value
    import torch
    import torch.distributed as dist
    t = torch.tensor([value], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(world, value: float) -> float:
    if world == 1:
        return value
    import torch
    import torch.distributed as dist
    t = torch.tensor([value], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(device), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=self.file, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        self.proc.wait()
        self.file.flush()
        self.file.seek(0)
        rows = [r.split(",") for r in self.file.read().splitlines() if r.strip()]
        os.unlink(self.file.name)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            r = [x.strip() for x in r]
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
            except (ValueError, IndexError):
                continue
            for name, flag in zip(names, r[5:9]):
                if flag.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def algorithmic_work(system):
    """Algorithmic flops per launch of the pair kernel, counted per unordered
    in-cutoff pair as the reference loops do (geometry 21, LJ body + epilogue
    36, real-space Coulomb body + epilogue 35), and per (k, atom) of the Ewald
    field (21) and rho (16) kernels."""
    import numpy as np
    p0 = system.pair_set(0)
    p1 = system.pair_set(1)
    key = lambda a: a[:, 0].astype(np.int64) * system.size + a[:, 1]
    union = np.union1d(key(p0), key(p1)).size if len(p0) or len(p1) else 0
    pair_flops = 21 * union + 36 * len(p0) + 35 * len(p1)
    nk = 0
    if system.coulomb is not None and hasattr(system.coulomb, "kmax"):
        nk = count_kvectors(system.cell.lengths, system.coulomb.kmax)
    return {"pairs_lj": int(len(p0)), "pairs_coulomb": int(len(p1)), "pair_flops": int(pair_flops),
            "kvectors": nk, "field_flops": 21 * nk * system.size, "rho_flops": 16 * nk * system.size}


def count_kvectors(lengths, kmax):
    """Size of the k-vector list of Ewald::prepare (ewald.rs:130-183, 353-379)."""
    k1 = [2.0 * math.pi / L for L in lengths]
    mx = max(k1) * kmax
    kmax2 = 1.0001 * mx * mx
    n = 0
    ranges = [((1, kmax), (-kmax, kmax), (-kmax, kmax)), ((0, 1), (1, kmax), (-kmax, kmax)),
              ((0, 1), (0, 1), (1, kmax))]
    for rx, ry, rz in ranges:
        for a in range(*rx):
            for b in range(*ry):
                for c in range(*rz):
                    k2 = (k1[0] * a) ** 2 + (k1[1] * b) ** 2 + (k1[2] * c) ** 2
                    if k2 <= kmax2:
                        n += 1
    return n


# MD steps a serving lane runs between admissions
SERVING_CHUNK = 64


def traffic_from_profiles(kernel: str):
    """DRAM bytes per launch of `kernel` from the committed ncu summary, if any."""
    path = os.path.join(ROOT, "profiles", "traffic.txt")
    if not os.path.exists(path):
        return None
    for line in open(path):
        parts = line.split()
        if len(parts) >= 2 and parts[0] == kernel:
            try:
                return float(parts[1])
            except ValueError:
                return None
    return None


def cpu_baseline(system, dt, seconds: float = 12.0):
    """The oracle's Velocity-Verlet on the host cores, on a bounded sample of
    steps of the same workload."""
    import numpy as np
    import oracle
    orc = oracle.Oracle(system)
    threads = oracle.num_threads()
    x, v = system.positions.copy(), system.velocities.copy()
    a = np.zeros_like(x)
    x, v, a = orc.velocity_verlet(x, v, a, dt, 1)  # warm-up step
    steps, t0 = 0, time.perf_counter()
    while True:
        x, v, a = orc.velocity_verlet(x, v, a, dt, 1)
        steps += 1
        el = time.perf_counter() - t0
        if el > seconds or steps >= 2000:
            break
    return {"value": system.size * steps / el, "unit": METRIC, "cores": threads, "kind": "port",
            "sample": f"{steps} Velocity-Verlet steps of the same {system.size}-atom system "
                      f"(O(N^2) forces, C++ restatement of lumol-core, OpenMP {threads} threads)"}


def run_reference(args, world, rank):
    if rank != 0:
        return
    import numpy as np
    import oracle
    oracle.build()
    if args.workload == "lj_batch":
        md_sys, md_p, mc_sys, mc_p, desc = batch_workload(args, "fp64")
        ref = reference_batch_steps(md_sys, md_p, mc_sys, mc_p, args.steps, args.warmup)
        md_atoms = sum(s.size for s in md_sys)
        mc_atoms = sum(s.size for s in mc_sys)
        value = ref["value"]
        base = {"value": value, "unit": METRIC, "cores": ref["threads"], "kind": "port",
                "sample": f"{args.steps} whole batched steps after {args.warmup} warm-up steps: one "
                          f"Velocity-Verlet + Berendsen step of each of the {len(md_sys)} MD replicas (O(N^2) "
                          f"forces) and one Translate move of each of the {len(mc_sys)} Monte Carlo chains "
                          f"(EnergyCache move cost and update); C++ restatement of lumol-core, OpenMP "
                          f"{ref['threads']} threads"}
        line = {"impl": "reference", "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": 0,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": ref["ms_per_step"],
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic (seeded replicas, lattice + jitter, Maxwell-Boltzmann velocities)",
                "config": batch_config(desc, md_atoms, mc_atoms, len(mc_sys)),
                "run": {"precision": "fp64", "parallelism": f"host, OpenMP {ref['threads']} threads",
                        "timed_iteration": "1 batched step (every MD replica, then every chain)"},
                "mc_moves_per_s": ref["mc_moves_per_s"], "md_atom_steps_per_s": ref["md_value"],
                "cpu_baseline": base,
                "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return
    system, dt, desc = make_system(args.workload, "fp64", args.cells)
    orc = oracle.Oracle(system)
    threads = oracle.num_threads()
    x, v = system.positions.copy(), system.velocities.copy()
    a = np.zeros_like(x)
    for _ in range(args.warmup):
        x, v, a = orc.velocity_verlet(x, v, a, dt, 1)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        x, v, a = orc.velocity_verlet(x, v, a, dt, 1)
    el = time.perf_counter() - t0
    value = system.size * args.steps / el
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": 0,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded lattice + Maxwell-Boltzmann velocities)",
        "config": {"workload": desc, "atoms": system.size, "precision": "fp64"},
        "cpu_baseline": {"value": value, "unit": METRIC, "cores": threads, "kind": "port",
                         "sample": f"{args.steps} timed Velocity-Verlet steps after {args.warmup} warm-up steps; "
                                   "C++ restatement of lumol-core's O(N^2) CPU path (the Rust reference has "
                                   "no toolchain here)"},
        "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def batch_config(desc, md_atoms, mc_atoms, mc_chains):
    """The workload of the batched-replica line, the same in both arms."""
    return {"workload": desc, "atoms": md_atoms + mc_atoms, "md_atoms": md_atoms, "mc_chains": mc_chains}


def reference_batch_steps(md_sys, md_p, mc_sys, mc_p, steps: int, warmup: int):
    """The reference's algorithm on the host cores for whole batched steps of
    the batched-replica workload: per step, one Velocity-Verlet step with the
    Berendsen thermostat of every MD replica (O(N^2) forces,
    lumol-sim/src/md/integrators.rs:44-69, md/thermostats.rs:112-121), then one
    Translate move of every Monte Carlo chain (a uniform displacement of one
    random atom, EnergyCache::move_molecule_cost and the Metropolis test,
    EnergyCache::update on acceptance; sys/cache.rs:118-220,
    mc/moves/translate.rs:41-125).  The caches are initialised before the
    timing.  The units counted are the GPU arm's: MD atoms + chains per step."""
    import numpy as np
    import oracle
    from lumol_gb300.units import K_BOLTZMANN
    threads = oracle.num_threads()
    md_orc = [oracle.Oracle(s) for s in md_sys]
    md_state = [(s.positions.copy(), s.velocities.copy(), np.zeros((s.size, 3))) for s in md_sys]
    md_temp = [t for _, (n, rho, t) in md_p]
    mc_orc = [oracle.Oracle(s) for s in mc_sys]
    mc_pos = [s.positions.copy() for s in mc_sys]
    import concurrent.futures
    with concurrent.futures.ThreadPoolExecutor(max_workers=max(1, threads)) as pool:
        list(pool.map(lambda o: o.cache_init(), mc_orc))  # EnergyCache::init, O(N^2) per chain, untimed
    mc_beta = [1.0 / (K_BOLTZMANN * t) for _, (n, rho, t) in mc_p]
    rng = np.random.default_rng(99)
    half = 0.3 / math.sqrt(3.0)
    md_time = mc_time = 0.0

    def one_step():
        nonlocal md_time, mc_time
        t0 = time.perf_counter()
        for k, o in enumerate(md_orc):
            x, v, a = md_state[k]
            md_state[k] = o.velocity_verlet(x, v, a, 1.0, 1, md_temp[k], 100.0)
        t1 = time.perf_counter()
        for k, o in enumerate(mc_orc):
            pos = mc_pos[k]
            i = int(rng.integers(len(pos)))
            newpos = pos[i:i + 1] + rng.uniform(-half, half, size=(1, 3))
            cost = mc_beta[k] * o.move_molecule_cost(i, newpos)
            if cost <= 0.0 or rng.random() < math.exp(-cost):
                pos[i] = newpos[0]  # (the wrap of the centre of mass does not change energies)
                o.set_positions(pos)
                o.cache_update()
        t2 = time.perf_counter()
        md_time += t1 - t0
        mc_time += t2 - t1
        return t2 - t0

    for _ in range(warmup):
        one_step()
    md_time = mc_time = 0.0
    total = sum(one_step() for _ in range(steps))
    md_atoms = sum(s.size for s in md_sys)
    return {"value": (md_atoms + len(mc_sys)) * steps / total, "ms_per_step": 1e3 * total / steps,
            "md_value": md_atoms * steps / md_time, "mc_moves_per_s": len(mc_sys) * steps / mc_time,
            "threads": threads}


def batch_workload(args, precision):
    """The batched-replica workload: seeded argon-type replicas, even indices
    run NVT MD (Velocity-Verlet dt = 1 fs, Berendsen tau = 100 steps), odd
    indices NVT Monte Carlo (Translate, delta = 0.3 A)."""
    from lumol_gb300 import workloads
    params, redraws = workloads.lj_replica_parameters(args.replicas)
    md_p = [(i, p) for i, p in enumerate(params) if i % 2 == 0]
    mc_p = [(i, p) for i, p in enumerate(params) if i % 2 == 1]
    md = [workloads.lj_replica(n, rho, t, 1000 + i, precision) for i, (n, rho, t) in md_p]
    mc = [workloads.lj_replica(n, rho, t, 1000 + i, precision) for i, (n, rho, t) in mc_p]
    desc = (f"{len(params)} argon-type LJ replicas (N ~ U{{64..4096}}, rho* ~ U(0.3,0.9), T ~ U(90,300) K, "
            f"seeded; {redraws} draw(s) with L < 2 rc redrawn), shifted LJ rc = 2.5 sigma; {len(md)} NVT MD "
            f"(VV dt=1 fs, Berendsen tau=100 fs) + {len(mc)} NVT MC (Translate delta=0.3 A); "
            f"one batched step = one Lumol step of every replica (MD: N atom-steps, MC: 1 move)")
    return md, md_p, mc, mc_p, desc


def timed_batch(args, world, local, precision: str, steps: int, warmup: int):
    """Builds the batched-replica workload at `precision` and times `steps`
    batched steps (MD half and MC half concurrently, on the two engines' own
    streams) with CUDA events; returns the figures and the live engines."""
    import concurrent.futures
    import ctypes

    import torch

    from lumol_gb300.batch import Batch

    md_sys, md_p, mc_sys, mc_p, desc = batch_workload(args, precision)
    md = Batch(md_sys, precision=precision, threads_per_atom=args.threads_per_atom)
    md.md_setup([1.0] * len(md_sys), [(t, 100.0) for _, (n, rho, t) in md_p])
    # a 2 A skin for the chains: fewer list rebuilds for single-particle moves of up to 0.3 A
    mc = Batch(mc_sys, precision=precision, skin=2.0)
    mc.md_setup([1.0] * len(mc_sys))
    for s, (i, (n, rho, t)) in enumerate(mc_p):
        mc.mc_setup(s, t, 0.3, 5000 + i)

    def stream_of(batch):
        ptr = ctypes.c_void_p()
        batch.engine.call("lg_get_stream", ctypes.byref(ptr))
        return torch.cuda.ExternalStream(ptr.value)

    s_md, s_mc = stream_of(md), stream_of(mc)
    chunk = max(1, min(args.chunk, steps))
    iters = (steps + chunk - 1) // chunk
    pool = concurrent.futures.ThreadPoolExecutor(max_workers=2)

    def one_iteration(steps_k):
        f1 = pool.submit(md.md_run, steps_k)
        f2 = pool.submit(mc.mc_run, steps_k)
        f1.result()
        f2.result()

    for _ in range(max(warmup, 3)):
        one_iteration(chunk)
    if steps % chunk:
        one_iteration(steps % chunk)
    torch.cuda.synchronize()
    n0a, n0b = ctypes.c_uint64(), ctypes.c_uint64()
    md.engine.call("lg_launch_count", ctypes.byref(n0a))
    mc.engine.call("lg_launch_count", ctypes.byref(n0b))
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(iters)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(iters)]
    mc_done = [torch.cuda.Event() for _ in range(iters)]
    barrier(world)
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    done = 0
    for k in range(iters):
        steps_k = min(chunk, steps - done)
        starts[k].record(s_md)
        s_mc.wait_event(starts[k])
        one_iteration(steps_k)
        mc_done[k].record(s_mc)
        s_md.wait_event(mc_done[k])
        ends[k].record(s_md)
        done += steps_k
    torch.cuda.synchronize()
    barrier(world)
    clk = clocks.stop()
    n1a, n1b = ctypes.c_uint64(), ctypes.c_uint64()
    md.engine.call("lg_launch_count", ctypes.byref(n1a))
    mc.engine.call("lg_launch_count", ctypes.byref(n1b))
    pool.shutdown()
    ms = sum(s.elapsed_time(e) for s, e in zip(starts, ends))
    ms_max = max_over_ranks(world, ms)
    work = (md.atoms + len(mc_sys)) * steps
    value = sum_over_ranks(world, float(work)) / (ms_max * 1e-3)
    return {"value": value, "ms_max": ms_max, "chunk": chunk, "clocks": clk, "desc": desc,
            "launches": int(n1a.value - n0a.value + n1b.value - n0b.value), "md": md, "mc": mc,
            "md_sys": md_sys, "md_p": md_p, "mc_sys": mc_sys, "mc_p": mc_p}


def main_batch(args, world, rank, local):
    import time as _time

    import torch

    from lumol_gb300 import _capi as C

    torch.cuda.set_device(local)
    leg = timed_batch(args, world, local, args.precision, args.steps, args.warmup)
    md, mc = leg["md"], leg["mc"]
    md_atoms, mc_chains = md.atoms, len(leg["mc_sys"])

    # MC chains alone, over many moves: moves/s of the MC half
    torch.cuda.synchronize()
    t0 = _time.perf_counter()
    mc.mc_run(2048)
    torch.cuda.synchronize()
    mc_rate = mc_chains * 2048 / (_time.perf_counter() - t0)

    # end to end: every step, all MD replicas' positions and velocities go
    # host -> device and back through the public calls (pinned buffers)
    e2e = None
    if not args.no_e2e:
        n_all = md_atoms
        pos = torch.empty((n_all, 3), dtype=torch.float64, pin_memory=True)
        vel = torch.empty((n_all, 3), dtype=torch.float64, pin_memory=True)
        md.engine.call("lg_md_get_state_all", C.dptr(pos.numpy()), C.dptr(vel.numpy()), None)
        steps_e2e = min(args.steps, 32)
        torch.cuda.synchronize()
        t0 = _time.perf_counter()
        for _ in range(steps_e2e):
            md.engine.call("lg_md_set_state_all", C.dptr(pos.numpy()), C.dptr(vel.numpy()), None)
            md.engine.call("lg_md_run", 1)
            md.engine.call("lg_md_get_state_all", C.dptr(pos.numpy()), C.dptr(vel.numpy()), None)
        torch.cuda.synchronize()
        el = max_over_ranks(world, _time.perf_counter() - t0)
        e2e = {"value": sum_over_ranks(world, float(n_all)) * steps_e2e / el, "unit": METRIC,
               "h2d_bytes_per_step": 2 * 3 * 8 * n_all, "d2h_bytes_per_step": 2 * 3 * 8 * n_all,
               "scope": "MD half (the MC chains' state stays on the device)"}

    roofline = None if args.no_roofline else batch_roofline(args, md, C)
    md.engine.close()
    mc.engine.close()

    # the plain FP64 path on the same workload: the mixed-vs-FP64 ratio of the metric
    fp64_leg = None
    if args.precision == "mixed" and not args.no_fp64_leg:
        steps64 = min(args.steps, 64)
        leg64 = timed_batch(args, world, local, "fp64", steps64, 3)
        leg64["md"].engine.close()
        leg64["mc"].engine.close()
        fp64_leg = {"value": leg64["value"], "unit": METRIC, "steps": steps64,
                    "ms_per_step": leg64["ms_max"] / steps64, "mixed_over_fp64": leg["value"] / leg64["value"]}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = batch_cpu_baseline(leg["md_sys"], leg["mc_sys"], leg["mc_p"])
    configs = None
    if rank == 0 and world == 1 and not args.no_configs:
        configs = config_legs(args, local)
    acc = None
    if rank == 0 and args.precision == "mixed" and not args.no_accuracy:
        from lumol_gb300 import workloads
        sub = leg["md_p"][:8]
        pairs = [(workloads.lj_replica(n, rho, t, 1000 + i, "fp64"),
                  workloads.lj_replica(n, rho, t, 1000 + i, "mixed")) for i, (n, rho, t) in sub]
        acc = accuracy_report(pairs, [1.0] * len(pairs), 2000,
                              f"the first {len(pairs)} MD replicas ({sum(p[0].size for p in pairs)} atoms), "
                              "starting positions + 0.05 A seeded jitter; NVE dt = 1 fs")
    if rank == 0:
        line = {
            "metric": METRIC, "value": leg["value"], "unit": METRIC, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": leg["ms_max"] / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64" if args.precision == "fp64" else "f32+f64",
            "data": "synthetic (seeded replicas, lattice + jitter, Maxwell-Boltzmann velocities)",
            "config": batch_config(leg["desc"], md_atoms, mc.atoms, mc_chains),
            "run": {"precision": args.precision,
                    "parallelism": f"replicas x{world}" if world > 1 else "one GPU, two engine streams",
                    "timed_iteration": f"{leg['chunk']} batched steps (lg_md_run || lg_mc_run)",
                    "l2": "inputs larger than L2 (neighbour lists of all replicas), no flush"},
            "fp64_plain": fp64_leg,
            "configs": configs,
            "accuracy": acc,
            "mc_moves_per_s": mc_rate,
            "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e,
            "gpu_launches": leg["launches"],
            "clocks": leg["clocks"],
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def main_serving(args, world, rank, local):
    """The serving stream: Poisson arrivals of LJ / NaCl+Ewald / water MD
    requests served by the continuous-batching server; throughput over the
    wall-clock span of the stream and p50 / p99 completion latency."""
    import torch

    from lumol_gb300 import workloads
    from lumol_gb300.serving import Server, latency_percentiles

    torch.cuda.set_device(local)
    requests = workloads.serving_requests(count=args.requests, rate=args.rate, seed=77 + rank,
                                          precision=args.precision)
    warm = workloads.serving_requests(count=4, rate=1000.0, seed=1, precision=args.precision, scale=0.02)
    server = Server(precision=args.precision, chunk=SERVING_CHUNK, max_lanes=4)
    server.run(warm)
    server.close()
    server = Server(precision=args.precision, chunk=SERVING_CHUNK, max_lanes=4)
    barrier(world)
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    t0 = time.perf_counter()
    done = server.run(requests)
    torch.cuda.synchronize()
    span = max_over_ranks(world, time.perf_counter() - t0)
    clk = clocks.stop()
    server.close()
    atom_steps = sum(r.system.size * r.nsteps for r in done)
    value = sum_over_ranks(world, float(atom_steps)) / span
    p50, p99 = latency_percentiles(done)
    kinds = {k: sum(1 for r in done if r.kind == k) for k in ("lj", "nacl", "water")}
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": len(done),
            "warmup": 4, "ms_per_step": None, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if args.precision == "fp64" else "f32+f64",
            "data": "synthetic (seeded Poisson request stream)",
            "config": {"workload": f"serving stream of {len(done)} MD requests at {args.rate}/s: "
                                   f"60% LJ (200-20000 atoms), 25% NaCl+Ewald (216-8000 ions), 15% water "
                                   f"(300-3000 molecules), 500-5000 steps each", "kinds": kinds,
                       "precision": args.precision, "timing": "host wall clock over the stream (latency metric)",
                       "lanes_max": server.stats.max_lanes, "lanes_opened": server.stats.lanes_opened,
                       "joins": server.stats.joins, "leaves": server.stats.leaves,
                       "chunks": server.stats.chunks},
            "latency_s": {"p50": p50, "p99": p99},
            "clocks": clk,
        }
        print(json.dumps(line), flush=True)


def time_md_device(system, steps: int, chunk: int = 16):
    """atom-steps/s of `steps` MD steps of one system with its state resident
    in HBM (lg_md_run of `chunk` steps per timed iteration, CUDA events on the
    engine's stream, the L2 flushed before every iteration)."""
    import ctypes

    import torch

    eng = system.engine()
    ptr = ctypes.c_void_p()
    eng.call("lg_get_stream", ctypes.byref(ptr))
    stream = torch.cuda.ExternalStream(ptr.value)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    for _ in range(3):
        eng.call("lg_md_run", chunk)
    torch.cuda.synchronize()
    ms, done = 0.0, 0
    while done < steps:
        k = min(chunk, steps - done)
        flush.zero_()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        eng.call("lg_md_run", k)
        e1.record(stream)
        e1.synchronize()
        ms += e0.elapsed_time(e1)
        done += k
    return system.size * steps / (ms * 1e-3)


def time_md_e2e(system, steps: int, every: int):
    """atom-steps/s through the reference-facing call, one Lumol step per call
    (Integrator::integrate -> lg_md_propagate on page-locked host arrays),
    the state copied back to the host every `every` steps (1: every step, as
    lg_md_integrate); host wall clock."""
    import torch

    from lumol_gb300 import _capi as C
    eng = system.engine()
    pos = torch.empty((system.size, 3), dtype=torch.float64, pin_memory=True)
    vel = torch.empty((system.size, 3), dtype=torch.float64, pin_memory=True)
    eng.call("lg_md_get_state", 0, C.dptr(pos.numpy()), C.dptr(vel.numpy()))
    px, pv = C.dptr(pos.numpy()), C.dptr(vel.numpy())
    for _ in range(3):
        eng.call("lg_md_propagate", px, pv, 1, C.LG_SYNC_DOWNLOAD)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k in range(steps):
        flags = C.LG_SYNC_DOWNLOAD if (k + 1) % every == 0 else 0
        eng.call("lg_md_propagate", px, pv, 1, flags)
    torch.cuda.synchronize()
    el = time.perf_counter() - t0
    return system.size * steps / el


def config_legs(args, local):
    """The single-system workloads (argon LJ 500 atoms, NaCl Ewald 1000 ions,
    water 5184 atoms) and the serving stream, each measured briefly: device
    atom-steps/s of the plain FP64 and the mixed path, end to end through
    lg_md_integrate (state copied back every step) and through
    lg_md_propagate at an output cadence of 10 steps, the mixed path's error
    against FP64 (force RMS, energy) with the NVE drift of both paths over the
    workload's stated run length, and the oracle on the host cores."""
    import torch

    import lumol_gb300 as lg
    torch.cuda.set_device(local)
    out = {}
    specs = {"argon": ("C0", 1000, 64), "nacl_ewald": ("C1", 2000, 64), "water": ("C2", 5000, 32)}
    for name, (tag, nve, steps) in specs.items():
        leg = {}
        for precision in ("fp64", "mixed"):
            system, dt, desc = make_system(name, precision)
            md = lg.MolecularDynamics(lg.VelocityVerlet(dt))
            md.setup(system)
            leg[f"{precision}_value"] = time_md_device(system, steps)
            if precision == "mixed":
                leg["e2e_every_step"] = time_md_e2e(system, 64, 1)
                leg["e2e_every_10_steps"] = time_md_e2e(system, 64, 10)
            system.engine().close()
        leg["mixed_over_fp64"] = leg["mixed_value"] / leg["fp64_value"]
        leg["workload"] = desc
        pair = (make_system(name, "fp64")[0], make_system(name, "mixed")[0])
        acc = accuracy_report([pair], [dt], nve, "starting positions + 0.05 A seeded jitter; NVE")
        leg.update({k: acc[k] for k in ("force_rms_rel", "energy_rel", "virial_rel", "nve_steps",
                                        "nve_drift_rel_fp64", "nve_drift_rel_mixed")})
        cpu = cpu_baseline(make_system(name, "fp64")[0], dt, seconds=3.0)
        leg["cpu_oracle"] = cpu["value"]
        leg["cpu_cores"] = cpu["cores"]
        leg["e2e_every_step_over_cpu"] = leg["e2e_every_step"] / cpu["value"]
        out[tag] = leg
    # C4: the seeded serving stream (48 requests at 40/s)
    from lumol_gb300 import workloads
    from lumol_gb300.serving import Server, latency_percentiles
    warm = workloads.serving_requests(count=4, rate=1000.0, seed=1, precision="mixed", scale=0.02)
    server = Server(precision="mixed", chunk=64, max_lanes=4)
    server.run(warm)
    server.close()
    requests = workloads.serving_requests(count=48, rate=40.0, seed=77, precision="mixed")
    server = Server(precision="mixed", chunk=64, max_lanes=4)
    t0 = time.perf_counter()
    done = server.run(requests)
    span = time.perf_counter() - t0
    server.close()
    p50, p99 = latency_percentiles(done)
    out["C4"] = {"value": sum(r.system.size * r.nsteps for r in done) / span, "unit": METRIC,
                 "requests": len(done), "rate_per_s": 40.0, "latency_s": {"p50": p50, "p99": p99},
                 "span_s": span, "lanes_max": server.stats.max_lanes, "joins": server.stats.joins,
                 "leaves": server.stats.leaves, "failed": server.stats.failed,
                 "lane_host_s": {"join": server.stats.join_s, "run": server.stats.run_s,
                                 "boundary": server.stats.boundary_s},
                 "workload": "seeded Poisson stream: 60% LJ (200-20000 atoms), 25% NaCl+Ewald (216-8000 ions), "
                             "15% water (300-3000 molecules), 500-5000 steps each, mixed precision"}
    return out


def batch_roofline(args, md, C):
    """Pair kernel of the MD half: algorithmic FLOP/s (21 geometry + 36 LJ per
    unordered in-cutoff pair, counted with lg_pairset over every replica) over
    its CUDA-event time, against the measured FMA peak of its pipe."""
    import ctypes
    kt = (ctypes.c_double * 8)()
    md.engine.call("lg_kernel_times", 10, kt)
    times = {name: kt[i] for i, name in enumerate(C.LG_KT_NAMES)}
    pairs = 0
    for s, system in enumerate(md.systems):
        pos, _ = md.state(s)
        count = ctypes.c_int64()
        md.engine.call("lg_pairset", s, C.dptr(pos), 0, None, 0, ctypes.byref(count))
        pairs += count.value
    flops = 57 * pairs
    fp64 = args.precision == "fp64"
    peak = ctypes.c_double()
    C.check(C.load().lg_fma_peak(1 if fp64 else 0, ctypes.byref(peak)))
    peak_source = (("FP64" if fp64 else "FP32") + " FMA throughput measured live by lg_fma_peak "
                   "(MEASURED_PEAKS.json has no such figure; no tensor cores on this path)")
    cluster, groups = ctypes.c_int32(), ctypes.c_int32()
    md.engine.call("lg_md_plan", ctypes.byref(cluster), ctypes.byref(groups))
    if cluster.value > 0:
        # the persistent kernel runs the whole step: time launches of the timed
        # iteration's length (up to 256 steps, one launch) with CUDA events on
        # the engine's stream (state advances, as in a run)
        import torch
        ptr = ctypes.c_void_p()
        md.engine.call("lg_get_stream", ctypes.byref(ptr))
        st = torch.cuda.ExternalStream(ptr.value)
        nst = max(8, min(args.chunk, args.steps, 256))
        md.md_run(nst)
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(3)]
        for e0, e1 in ev:
            e0.record(st)
            md.md_run(nst)
            e1.record(st)
        torch.cuda.synchronize()
        ms = min(e0.elapsed_time(e1) for e0, e1 in ev)
        achieved = flops * nst / (ms * 1e-3) / 1e12
        per_step = traffic_from_profiles("md_persist_kernel_lj_batch256_per_step")
        return {"bound": "fp32", "achieved": achieved, "peak": peak.value, "unit": "TFLOP/s",
                "frac": achieved / peak.value, "traffic": per_step * nst if per_step else None,
                "kernel": "md_persist_kernel", "kernel_ms": ms, "steps_per_launch": nst,
                "cluster": cluster.value, "groups": groups.value,
                "includes": "whole MD steps: integration, list rebuilds, forces, thermostat",
                "peak_source": peak_source, "kernel_ms_by_group": times,
                "work": {"pairs_lj": pairs, "pair_flops_per_step": flops}}
    achieved = flops / (times["pair"] * 1e-3) / 1e12
    kernel = "pair_half_kernel" if fp64 else "pair_mixed_kernel"
    return {"bound": "fp64" if fp64 else "fp32", "achieved": achieved, "peak": peak.value, "unit": "TFLOP/s",
            "frac": achieved / peak.value,
            "traffic": traffic_from_profiles(kernel + "_lj_batch256" + ("_sorted" if not fp64 else "")),
            "kernel": kernel, "kernel_ms": times["pair"], "peak_source": peak_source,
            "kernel_ms_by_group": times, "work": {"pairs_lj": pairs, "pair_flops": flops}}


def accuracy_report(pairs, timesteps, nve_steps: int, label: str):
    """Error of the mixed path against the plain FP64 path, stated per
    workload: for each (FP64, mixed) pair of the same seeded system, the
    relative force RMS sqrt(sum|F_mixed - F_fp64|^2 / sum|F_fp64|^2), the
    relative potential-energy error, the virial error relative to its largest
    entry, all at the starting positions; then both paths run `nve_steps`
    Velocity-Verlet steps without thermostat and the total-energy drift
    |E(end) - E(0)| / |E(0)| is reported for each.  Maxima over the pairs."""
    import numpy as np

    from lumol_gb300 import units
    from lumol_gb300.batch import Batch

    out = {"vs": "plain FP64 GPU path on the same seeded systems", "systems": label,
           "force_rms_rel": 0.0, "energy_rel": 0.0, "virial_rel": 0.0, "nve_steps": nve_steps}
    # the same seeded 0.05 A jitter on both copies: a perfect lattice has zero
    # forces by symmetry, which would make the relative force error meaningless
    rng = np.random.default_rng(4242)
    for sd, sm in pairs:
        d = rng.uniform(-0.05, 0.05, size=(sd.size, 3))
        sd.positions = sd.positions + d
        sm.positions = sm.positions + d
    def worst(a, b):  # max that keeps a NaN visible (Python's max drops it)
        return b if (b != b or b > a) else a

    for sd, sm in pairs:
        fd, ed, wd = sd.compute()
        fm, em, wm = sm.compute()
        out["force_rms_rel"] = worst(out["force_rms_rel"], float(np.sqrt(np.sum((fm - fd) ** 2) / np.sum(fd ** 2))))
        out["energy_rel"] = worst(out["energy_rel"], abs(em - ed) / abs(ed))
        out["virial_rel"] = worst(out["virial_rel"], float(np.max(np.abs(wm - wd)) / np.max(np.abs(wd))))
    for name, idx in (("fp64", 0), ("mixed", 1)):
        systems = [p[idx] for p in pairs]
        b = Batch(systems, precision=name)
        b.md_setup(timesteps)
        e0 = []
        for s, system in enumerate(systems):
            _, v = b.state(s)
            e0.append(b.energy(s) + 0.5 * float(np.sum(system.masses[:, None] * v * v)))
        b.md_run(nve_steps)
        drift, per_atom = 0.0, 0.0
        for s, system in enumerate(systems):
            _, v = b.state(s)
            e1 = b.energy(s) + 0.5 * float(np.sum(system.masses[:, None] * v * v))
            drift = worst(drift, abs(e1 - e0[s]) / abs(e0[s]))
            per_atom = worst(per_atom, units.to(abs(e1 - e0[s]), "kJ/mol") / system.size)
        b.engine.close()
        out[f"nve_drift_rel_{name}"] = drift
        out[f"nve_drift_kJmol_per_atom_{name}"] = per_atom
    return out


def batch_cpu_baseline(md_sys, mc_sys, mc_p, seconds: float = 15.0):
    """The oracle on the host cores over a bounded sample of the same replicas:
    MD steps of MD replicas (O(N^2) forces) in round robin until `seconds`."""
    import numpy as np
    import oracle
    threads = oracle.num_threads()
    orcs = [oracle.Oracle(s) for s in md_sys]
    state = [(s.positions.copy(), s.velocities.copy(), np.zeros((s.size, 3))) for s in md_sys]
    atom_steps, steps, k = 0, 0, 0
    t0 = time.perf_counter()
    while time.perf_counter() - t0 < seconds:
        x, v, a = state[k]
        state[k] = orcs[k].velocity_verlet(x, v, a, 1.0, 1)
        atom_steps += md_sys[k].size
        steps += 1
        k = (k + 1) % len(md_sys)
    el = time.perf_counter() - t0
    return {"value": atom_steps / el, "unit": METRIC, "cores": threads, "kind": "port",
            "sample": f"{steps} Velocity-Verlet steps over the first {min(steps, len(md_sys))} MD replicas in "
                      f"round robin (O(N^2) C++ restatement of lumol-core, OpenMP {threads} threads)"}


def main():
    args = parse()
    world, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, world, rank)
        return
    if args.workload == "lj_batch":
        main_batch(args, world, rank, local)
        return
    if args.workload == "serving":
        main_serving(args, world, rank, local)
        return
    import ctypes

    import numpy as np
    import torch

    from lumol_gb300 import build as engine_build
    if not os.path.exists(engine_build.LIB):
        engine_build.build()
    import lumol_gb300 as lg
    from lumol_gb300 import _capi as C

    torch.cuda.set_device(local)
    system, dt, desc = make_system(args.workload, args.precision, args.cells)
    md = lg.MolecularDynamics(lg.VelocityVerlet(dt))
    md.setup(system)
    eng = system.engine()
    stream_ptr = ctypes.c_void_p()
    eng.call("lg_get_stream", ctypes.byref(stream_ptr))
    stream = torch.cuda.ExternalStream(stream_ptr.value)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")

    chunk = max(1, min(args.chunk, args.steps))
    iters = (args.steps + chunk - 1) // chunk
    for _ in range(max(args.warmup, 3)):
        eng.call("lg_md_run", chunk)
    if args.steps % chunk:
        eng.call("lg_md_run", args.steps % chunk)  # instantiate the remainder's graph outside the timing
    torch.cuda.synchronize()

    n0 = ctypes.c_uint64()
    eng.call("lg_launch_count", ctypes.byref(n0))
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(iters)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(iters)]
    barrier(world)
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    done = 0
    for k in range(iters):
        steps_k = min(chunk, args.steps - done)
        flush.zero_()
        torch.cuda.synchronize()
        starts[k].record(stream)
        eng.call("lg_md_run", steps_k)
        ends[k].record(stream)
        done += steps_k
    torch.cuda.synchronize()
    barrier(world)
    clk = clocks.stop()
    n1 = ctypes.c_uint64()
    eng.call("lg_launch_count", ctypes.byref(n1))
    ms = sum(s.elapsed_time(e) for s, e in zip(starts, ends))
    ms_max = max_over_ranks(world, ms)
    atoms_total = sum_over_ranks(world, float(system.size))
    value = atoms_total * args.steps / (ms_max * 1e-3)

    # end to end through the public call, pinned host buffers
    e2e = None
    bytes_state = 2 * 3 * 8 * system.size
    if not args.no_e2e:
        e2e = run_e2e(args, world, eng, C, torch, system, atoms_total, bytes_state)

    roofline = None if args.no_roofline else measure_roofline(args, eng, C, system)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(system, dt)
    acc = None
    if rank == 0 and args.precision == "mixed" and not args.no_accuracy:
        pair = (make_system(args.workload, "fp64", args.cells)[0], make_system(args.workload, "mixed", args.cells)[0])
        nve = {"nacl_ewald": 2000, "water": 5000}.get(args.workload, 1000)
        acc = accuracy_report([pair], [dt], nve, f"the benchmarked system, starting positions + 0.05 A seeded jitter; NVE dt = {dt} fs")

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64" if args.precision == "fp64" else "f32+f64",
            "data": "synthetic (seeded lattice + Maxwell-Boltzmann velocities)",
            "config": {"workload": desc, "atoms": system.size, "precision": args.precision,
                       "parallelism": f"replicas x{world}" if world > 1 else "single system",
                       "timed_iteration": f"lg_md_run of {chunk} MD steps",
                       "l2": "flushed before every timed iteration (256 MiB write)"},
            "roofline": roofline,
            "cpu_baseline": cpu,
            "e2e": e2e,
            "accuracy": acc,
            "gpu_launches": int(n1.value - n0.value),
            "clocks": clk,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def run_e2e(args, world, eng, C, torch, system, atoms_total, bytes_state):
    """The same metric through lg_md_integrate (Integrator::integrate), one MD
    step per call, positions and velocities copied from pinned host memory and
    back every step; host wall clock."""
    pos = torch.empty((system.size, 3), dtype=torch.float64, pin_memory=True)
    vel = torch.empty((system.size, 3), dtype=torch.float64, pin_memory=True)
    eng.call("lg_md_get_state", 0, C.dptr(pos.numpy()), C.dptr(vel.numpy()))
    for _ in range(3):
        eng.call("lg_md_integrate", C.dptr(pos.numpy()), C.dptr(vel.numpy()), 1)
    torch.cuda.synchronize()
    barrier(world)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        eng.call("lg_md_integrate", C.dptr(pos.numpy()), C.dptr(vel.numpy()), 1)
    torch.cuda.synchronize()
    e2e_s = max_over_ranks(world, time.perf_counter() - t0)
    return {"value": atoms_total * args.steps / e2e_s, "unit": METRIC, "h2d_bytes_per_step": bytes_state,
            "d2h_bytes_per_step": bytes_state}


def measure_roofline(args, eng, C, system):
    """Dominant force kernel: algorithmic FLOP/s (per-unit work x units per
    launch / CUDA-event time of one launch) against the measured FMA peak of
    the pipe it runs on (FP64 for the plain path, FP32 for the mixed one)."""
    import ctypes
    kt = (ctypes.c_double * 8)()
    eng.call("lg_kernel_times", 20, kt)
    times = {name: kt[i] for i, name in enumerate(C.LG_KT_NAMES)}
    work = algorithmic_work(system)
    fp64 = args.precision == "fp64"
    peak = ctypes.c_double()
    C.check(C.load().lg_fma_peak(1 if fp64 else 0, ctypes.byref(peak)))
    candidates = {"pair": work["pair_flops"], "field": work["field_flops"], "rho": work["rho_flops"]}
    dominant = max(candidates, key=lambda k: times.get(k, 0.0))
    achieved = candidates[dominant] / (times[dominant] * 1e-3) / 1e12
    names = {"pair": "pair_half_kernel" if fp64 else "pair_mixed_kernel",
             "field": "field_kernel" if fp64 else "field_mixed_kernel",
             "rho": "rho_kernel" if fp64 else "rho_mixed_kernel"}
    pipe = "FP64" if fp64 else "FP32"
    return {"bound": "fp64" if fp64 else "fp32", "achieved": achieved, "peak": peak.value, "unit": "TFLOP/s",
            "frac": achieved / peak.value, "traffic": traffic_from_profiles(names[dominant]),
            "kernel": names[dominant], "kernel_ms": times[dominant],
            "peak_source": f"{pipe} FMA throughput measured live by lg_fma_peak (MEASURED_PEAKS.json has no "
                           f"{pipe} figure; this path does not use tensor cores)",
            "kernel_ms_by_group": times, "work": work}



if __name__ == "__main__":
    main()
