#!/usr/bin/env python3
"""Benchmark of the per-time-step dengue simulation: agent-steps/s on the plain large workload.

Workload (synthetic, seeded): 1,000,000 humans and 6,000,000 mosquito slots in 2,500
communities on a 50x50 rook lattice, lognormal(0, 0.8) community sizes, 4 serotypes,
3,650 daily steps per run (arbo_gpu_fit_gb300.configs.plain_large).

A "step" is one simulation time step over the whole census (human and mosquito demographic
passes, force of infection with dispersal, infection draws, series row). ``value`` =
(humans + mosquito slots) * timed steps * ranks / max-over-ranks device time, with the census
resident in HBM. The census read per step (63 MB) is smaller than L2, so every timed step is
preceded by an untimed kernel that reads a 320 MiB buffer (cold L2 at each step start).

Arms:
  --impl ours (default): the sm_103a library through its C-ABI.
  --impl reference: the reference has no CPU path of its own; its per-step logic restated
      serially (oracle/, the parity checker) is run as independent replicas on all host cores.
Multi-GPU: replicas only (every rank runs its own simulation, different seed); gloo carries the
per-rank timings, no data-path collective.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

# Algorithmic bytes per agent-step of the demographic pass, the roofline figure: what the
# reference's algorithm moves per agent (read age 4 + death age 4 + status 1, write age 4).
BYTES_PER_AGENT_STEP = 13
# What this library's layout moves instead: ages are kept as birth times, so a mosquito slot costs
# its state byte and death time (5) and a human its next event time (4), and a survivor without a
# transition writes nothing; each birth writes the newborn's PLE, birth time and death time (12)
# and a status byte, plus the status byte of the death that freed its slot.
LAYOUT_BYTES_PER_HUMAN_STEP = 4
LAYOUT_BYTES_PER_SLOT_STEP = 5
LAYOUT_BYTES_PER_BIRTH = 14
FLUSH_MB = 320
PEAKS_FILE = ROOT / "MEASURED_PEAKS.json"
FALLBACK_HBM_GBS = 6800.0
# Per-launch DRAM traffic of the demographic kernel on this workload, from one ncu capture of a
# launch at step 5 (the command is kept with its summary under profiles/):
# dram__bytes_read.sum + dram__bytes_write.sum (42,747,136 + 8,205,824 bytes).
DEMOG_TRAFFIC_BYTES = 50_952_960


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3600)
    ap.add_argument("--warmup", type=int, default=50)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--flush-mb", type=int, default=FLUSH_MB)
    ap.add_argument("--cpu-steps", type=int, default=60, help="oracle steps timed for the CPU baseline")
    ap.add_argument("--e2e-runs", type=int, default=3)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--small", action="store_true", help="profile-sized workload (1/8 of the large one)")
    ap.add_argument("--batched-instances", type=int, default=256,
                    help="instances of the batched configuration measured beside the headline (0: skip)")
    ap.add_argument("--batched-steps", type=int, default=40)
    ap.add_argument("--ref-gpu-steps", type=int, default=-1,
                    help="steps of the reference's own CUDA kernels timed in the reference arm "
                         "(-1: the same as --steps after --warmup untimed steps; 0: skip)")
    return ap.parse_args()


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo", rank=rank, world_size=world)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def all_max(world, x: float) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def workload(args, seed, max_time=None):
    from arbo_gpu_fit_gb300 import configs
    T = max(3650, args.warmup + args.steps) if max_time is None else max_time
    if args.small:
        return configs.scaled(125_000, 750_000, 18, T, seed=seed)
    return configs.plain_large(seed=seed, max_time=T)


def config_block(w, args, world):
    sp = w.parameter.simulation
    return {
        "workload": ("plain_large: 1,000,000 humans + 6,000,000 mosquito slots, 2,500 communities "
                     "(50x50 rook CSR), lognormal(0,0.8) sizes, 4 serotypes, 3,650 steps/run")
        if not args.small else "plain_large shape at 1/8 scale (profiling)",
        "humans": int(sp.nSize), "mosquito_slots": int(sp.mSize), "communities": w.network.subPopTotal,
        "serotypes": int(sp.nStrains), "steps_per_run": 3650, "seed": w.seed,
        "l2": f"flushed before every timed step by reading a {args.flush_mb} MiB buffer (untimed)",
        "parallelism": f"replicas x{world} (no data-path collective)",
        "timing": "CUDA events around each graph-launched step on the launching stream",
    }


class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                                          "-i", str(self.device), "-lms", "20"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            time.sleep(0.3)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            time.sleep(0.1)
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                self.out, _ = self.proc.communicate()

    def summary(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = [r.split(",") for r in self.out.strip().splitlines() if r.count(",") >= 8]
        sm, smax, reasons, power = [], [], set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                smax.append(float(r[2]))
                power.append(float(r[3]))
            except ValueError:
                continue
            for name, v in zip(names, r[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(name)
        load = [s for s, p in zip(sm, power) if p > min(power) + 0.25 * (max(power) - min(power))] if power else []
        return {"sm_mhz": statistics.median(load or sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": sorted(reasons), "samples": len(sm)}


def hbm_peak():
    try:
        peaks = json.loads(PEAKS_FILE.read_text())
        return float(peaks["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def ref_workload(small, seed, max_time=3650):
    """The workload of the CPU legs, built without loading the library they are compared with
    (oracle/workloads.py; the profiling-sized case comes from the package's configs)."""
    if small:
        from arbo_gpu_fit_gb300 import configs
        return configs.scaled(125_000, 750_000, 18, max_time, seed=seed)
    from oracle import workloads
    return workloads.plain_large(seed=seed, max_time=max_time)


def run_oracle_sample(args_tuple):
    """One CPU replica: init (untimed) + `steps` oracle steps (timed). Runs in a spawned process."""
    steps, seed, small = args_tuple
    sys.path.insert(0, str(ROOT))
    from oracle.binding import OracleSim
    w = ref_workload(small, seed)
    o = OracleSim(w.parameter.simulation, w.network, w.n_sizes, w.m_sizes, w.max_time, w.seed)
    o.init()
    t0 = time.perf_counter()
    o.step(steps)
    dt = time.perf_counter() - t0
    return w.agents, steps, dt


def cpu_baseline(args, cores):
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    jobs = [(args.cpu_steps, 1000 + k, args.small) for k in range(cores)]
    with ctx.Pool(cores) as pool:
        res = pool.map(run_oracle_sample, jobs)
    agents = res[0][0]
    rate = sum(a * s / dt for a, s, dt in res)
    per_step_ms = statistics.mean(dt / s for _, s, dt in res) * 1e3
    return rate, per_step_ms, agents


def reference_arm(args, world, rank):
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    w = ref_workload(args.small, 20261203, max(3650, args.warmup + args.steps))
    rate, per_step_ms, agents = cpu_baseline(args, cores)
    sample = (f"{cores} independent replicas of the workload, each: init (untimed) + {args.cpu_steps} "
              f"serial steps (timed), oracle/ restatement of the reference's per-step logic")
    line = {
        "metric": "agent-steps/s", "value": rate, "unit": "agent-steps/s", "n_gpus": args.gpus,
        "steps": args.cpu_steps, "warmup": 0, "ms_per_step": per_step_ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic",
        "config": config_block(w, args, 1), "impl": "reference",
        "cpu_baseline": {"value": rate, "unit": "agent-steps/s", "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": rate, "unit": "agent-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference has no CPU implementation; its per-step logic restated serially in oracle/",
    }
    if args.ref_gpu_steps != 0:
        line["reference_cuda_kernels"] = reference_cuda_kernels(args, w)
    print(json.dumps(line), flush=True)


def reference_cuda_kernels(args, w):
    """The reference's own CUDA kernels on this GPU: compiled from its sources for sm_103a
    (oracle/ref_build.py) and launched as cpp/simulation.cpp launches them, dataCollect included
    (oracle/ref_kernels.py). Same workload shape; community sizes drawn by the reference's own
    assignment kernel with this workload's community weights. Reported beside the arm's CPU value."""
    from oracle import ref_build

    if not ref_build.prebuilt():
        return {"unavailable": "reference cubins not built (oracle/ref_build.py needs the reference sources)"}
    try:
        from tests.distribution import expected_series
        from oracle.ref_kernels import ReferenceKernels

        sp = w.parameter.simulation
        K = args.steps if args.ref_gpu_steps < 0 else args.ref_gpu_steps
        W = args.warmup
        ref = ReferenceKernels(0)
        ref.setup(sp, w.network.loc, w.network.to, w.network.weight, expected_series(sp, w.max_time),
                  int(sp.nSize), int(sp.mSize), w.max_time, int(sp.nStrains), n_weights=w.n_sizes, m_weights=w.m_sizes)
        ref.init(w.seed, collect=False)
        r = ref.time_steps(K, W)
        ref.drv.free_all()
        sec = r["device_ms"] / 1e3
        return {"value": w.agents * K / sec, "unit": "agent-steps/s", "ms_per_step": r["device_ms"] / K,
                "steps": K, "warmup": W, "launches_per_step": r["launches_per_step"],
                "timing": (f"steps recorded into CUDA graphs of {r['graph_steps']} steps, launched back to back "
                           "between CUDA events on the launching stream; L2 not flushed"),
                "kind": "reference CUDA kernels (sm_103a cubins from the reference sources)"}
    except Exception as e:  # noqa: BLE001
        return {"unavailable": f"{type(e).__name__}: {e}"[:300]}


def births_per_step(sim, W, K, samples=8):
    """Mean agents born (humans reborn, mosquito slots recruited) per step over steps W..W+K of a
    re-initialised run: an agent of age 0 in a census snapshot was born in the step just taken."""
    sim.init()
    sim.step(W)
    stride = max(K // samples, 1)
    total = 0
    for _ in range(samples):
        sim.step(stride)
        total += int((sim.census("n_age") == 0).sum())
        total += int(((sim.census("m_age") == 0) & (sim.census("m_dead") == 0)).sum())
    return total / samples


def ours_arm(args, world, rank, local):
    from arbo_gpu_fit_gb300 import _native
    from arbo_gpu_fit_gb300.simulation import Simulation, simulation

    lib = _native.load()
    _native.check(lib.arbo_set_device(local))
    seed = 20261203 + rank
    w = workload(args, seed)
    K, W = args.steps, args.warmup
    assert W >= 3, "at least 3 warm-up steps"

    # --- device throughput: K graph-launched steps, L2 flushed before each, CUDA events per step
    sim = Simulation(w.parameter, w.network, w.n_sizes, w.m_sizes, max_time=w.max_time, seed=w.seed)
    sim.init()
    sim.step(W)
    sim.status()  # synchronise
    barrier(world)
    with ClockSampler(local) as clocks:
        step_ms = sim.time_steps(K, args.flush_mb)
        sim.status()
    barrier(world)
    err, t_now = sim.status()
    if err:
        raise RuntimeError(f"device error word {err}")
    t_rank = float(step_ms.sum()) / 1e3
    t_max = all_max(world, t_rank)
    value = w.agents * K * world / t_max

    # --- per-kernel times over the same K steps (re-initialised, same seed), cold L2 per step
    sim.init()
    sim.step(W)
    phases = sim.time_phases(K, args.flush_mb)
    births = births_per_step(sim, W, K)
    sim.close()
    demog_ms = phases[0]
    peak, peak_kind = hbm_peak()
    achieved = BYTES_PER_AGENT_STEP * w.agents / (demog_ms * 1e-3) / 1e9
    humans = int(w.parameter.simulation.nSize)
    layout_bytes = (LAYOUT_BYTES_PER_HUMAN_STEP * humans + LAYOUT_BYTES_PER_SLOT_STEP * (w.agents - humans) +
                    LAYOUT_BYTES_PER_BIRTH * births)
    layout_gbs = layout_bytes / (demog_ms * 1e-3) / 1e9
    traffic = DEMOG_TRAFFIC_BYTES * (w.agents / 7_000_000) if DEMOG_TRAFFIC_BYTES else None

    # --- end to end: the reference-facing call with host buffers (create + upload, init, a full
    # 3,650-step run, series download, destroy), wall clock, no L2 flush
    e2e_w = workload(args, seed, max_time=3650)
    walls, io = [], (0, 0)
    for _ in range(args.e2e_runs):
        barrier(world)
        t0 = time.perf_counter()
        with Simulation(e2e_w.parameter, e2e_w.network, e2e_w.n_sizes, e2e_w.m_sizes, max_time=3650,
                        seed=e2e_w.seed) as s2:
            s2.init()
            s2.run()
            for k in ("n_incidence", "n_infected", "one_subpop", "n_count", "m_count"):
                s2.series(k)
            io = s2.io_bytes()
        walls.append(time.perf_counter() - t0)
    e2e_wall = all_max(world, statistics.median(walls)) if walls else None
    e2e_value = e2e_w.agents * 3650 * world / e2e_wall if walls else None

    if rank != 0:
        return
    step_gbs = BYTES_PER_AGENT_STEP * w.agents / (t_max / K) / 1e9
    line = {
        "metric": "agent-steps/s", "value": value, "unit": "agent-steps/s", "n_gpus": world, "steps": K,
        "warmup": W, "ms_per_step": t_max * 1e3 / K, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int32", "data": "synthetic", "config": config_block(w, args, world),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "kernel": "k_demog", "peak_kind": peak_kind,
                     "bytes_per_agent_step": BYTES_PER_AGENT_STEP, "kernel_ms": demog_ms,
                     "layout": {"bytes": layout_bytes, "bytes_per_human_step": LAYOUT_BYTES_PER_HUMAN_STEP,
                                "bytes_per_slot_step": LAYOUT_BYTES_PER_SLOT_STEP,
                                "bytes_per_birth": LAYOUT_BYTES_PER_BIRTH, "births_per_step": births,
                                "achieved": layout_gbs, "frac": layout_gbs / peak},
                     "phase_ms": {"demographic": phases[0], "foi_series": phases[1], "infection": phases[2],
                                  "step": phases[3]},
                     # The whole graph-launched step (all three kernels) in the same 13 B figure.
                     "step": {"achieved": step_gbs, "frac": step_gbs / peak, "ms": t_max * 1e3 / K}},
        "e2e": {"value": e2e_value, "unit": "agent-steps/s", "h2d_bytes_per_step": io[0] / 3650,
                "d2h_bytes_per_step": io[1] / 3650, "granularity": "one simulation() call per iteration: "
                "create+upload, init, 3,650 steps, series download; median of runs", "runs": len(walls),
                "wall_s": e2e_wall},
        "clocks": clocks.summary(),
        "gpu_launches": 4 * K + -(-K // 64),
        "gpu_launches_detail": {"step_kernels": 3 * K, "l2_flush_kernels": K, "step_counter_kernels": -(-K // 64)},
    }
    if args.batched_instances > 0:
        line["batched"] = batched_measure(args, seed)
    if world == 1 and not args.no_cpu_baseline:
        rate, per_step_ms, _ = cpu_baseline(args, 1)
        line["cpu_baseline"] = {"value": rate, "unit": "agent-steps/s", "cores": 1, "kind": "port",
                                "sample": f"init (untimed) + {args.cpu_steps} serial steps of the same workload, "
                                          f"oracle/ restatement on 1 host core ({per_step_ms:.0f} ms/step)"}
    print(json.dumps(line), flush=True)


def batched_measure(args, seed):
    """The batched configuration: independent instances of uneven sizes and parameters advanced by
    one persistent kernel per phase (arbo_batch_*), launch shapes picked by the autotuner, against
    the same instances stepped one at a time (one graph-launched handle after another). The working
    set is far larger than L2, so no flush is needed."""
    from arbo_gpu_fit_gb300 import configs
    from arbo_gpu_fit_gb300.simulation import Batch, Simulation

    ws = configs.batched(args.batched_instances, seed=seed)
    t0 = time.perf_counter()
    sims = [Simulation(w.parameter, w.network, w.n_sizes, w.m_sizes, max_time=w.max_time, seed=w.seed) for w in ws]
    create_s = time.perf_counter() - t0
    K = args.batched_steps
    with Batch(sims) as b:
        agents = b.agents
        b.init()
        arch, tuned_ms = b.autotune(2)
        b.step(3)
        step_ms = b.time_steps(K)
        phases = b.time_phases(5)
        grids = b.arch()[1]
    batched_s = float(step_ms.sum()) / 1e3
    # The same instances, one after another, each graph-launched (same step range: the batch left
    # every instance at the same step).
    seq_ms = 0.0
    for s in sims:
        seq_ms += float(s.time_steps(K).sum())
    for s in sims:
        s.close()
    return {
        "workload": (f"{len(ws)} instances: humans log-uniform [2e4, 2e6], 6 mosquito slots per human, communities "
                     "log-uniform [100, 4000] on near-square rook lattices, 4 serotypes, 1,825 steps/run, "
                     "parameters uniform in the MCMC prior box"),
        "instances": len(ws), "agents": agents, "steps": K,
        "value": agents * K / batched_s, "unit": "agent-steps/s", "ms_per_step": batched_s * 1e3 / K,
        "sequential_value": agents * K / (seq_ms / 1e3), "speedup_vs_sequential": (seq_ms / 1e3) / batched_s,
        "roofline_frac_step": BYTES_PER_AGENT_STEP * agents * K / batched_s / 1e9 / hbm_peak()[0],
        "phase_ms": {"demographic": phases[0], "foi_series": phases[1], "infection": phases[2], "step": phases[3]},
        "autotuned": {"demogBlock": arch.demogBlock, "demogUnroll": arch.demogUnroll, "foiBlock": arch.foiBlock,
                      "infectBlock": arch.infectBlock, "grids": grids, "phase_ms": tuned_ms.tolist()},
        "create_s": create_s,
        "timing": "CUDA events around each graph-launched batch step; no L2 flush (working set >> L2)",
    }


def main():
    args = parse()
    world, rank, local = dist_setup()
    if args.impl == "reference":
        reference_arm(args, world, rank)
    else:
        ours_arm(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
