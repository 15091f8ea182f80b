"""Benchmark: agent-steps/s of the UMANS per-step agent update on one GB300.

Workload (default): 100 000 agents uniform in a 400 x 400 m toric world,
SocialForcesAvoidance (range 5) + GoalReachingForce, gradient method, dt 0.1
(the plain large workload; synthetic seeded data).  A step is one
WorldBase::DoStep over all agents.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line.  `value` is device-resident throughput with the L2
cache flushed (a 256 MiB write) before every timed step; `e2e` is the same
metric through the reference-facing C functions (SetAgentPositions ->
DoSimulationSteps(1) -> GetAgentPositions) with host buffers.  Under
torchrun (N > 1) every rank runs an independent replica (the step has no
cross-scenario exchange) and rank 0 reports the aggregate.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "agent-steps/s plain vs batched, fwd+adjoint step time; 1 GB300 at stated tol"
L2_FLUSH_BYTES = 256 << 20
# algorithmic HBM bytes of the fused per-agent kernel, per agent-step:
# reads  self cell-sorted pos 8 + vel 8 + (pref, radius) 16 + slot 4,
#        parameters 16, goal 8, policy index 4          = 64 B
# writes pos 8, vel 8, velocity-without-forces 8, view 8 = 32 B
K_AGENT_BYTES_PER_AGENT = 96
# FP32 operations per neighbour pair, counted from the reference source
# (SocialForcesAvoidance.cpp:26-110 ~55, contact term policy.cpp:107-141 ~12),
# plus ~40 per agent (goal force, clamps, integration)
SF_FLOP_PER_PAIR = 67
SF_FLOP_PER_AGENT = 40


def workload(name: str, tmp: str):
    from umans_gb300 import scenarios as S
    if name == "socialforces_toric":
        sc = S.socialforces_toric()
        cfg = dict(workload="socialforces_toric", agents=100_000, world="toric 400x400 m",
                   policy="SocialForcesAvoidance(range 5)+GoalReachingForce, gradient", dt=0.1)
    elif name == "karamouzas_corridor":
        sc = S.karamouzas_corridor()
        cfg = dict(workload="karamouzas_corridor", agents=1_000_000, world="infinite, 10000x100 m corridor",
                   policy="Karamouzas(range 10), regular sampling 181 samples", dt=0.05)
    elif name == "circle_orca":
        sc = S.circle_orca()
        cfg = dict(workload="circle_orca", agents=50, world="infinite", policy="ORCA global", dt=0.1)
    else:
        raise SystemExit(f"unknown workload {name}")
    path = sc.write(os.path.join(tmp, name + ".xml"))
    return path, sc.n, cfg


class ClockSampler:
    """Samples SM clocks and throttle reasons with nvidia-smi while running."""

    def __init__(self, index: int = 0):
        self.index = index
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def __enter__(self):
        def run():
            q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
                 "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
                 "clocks_event_reasons.sw_power_cap")
            while not self._stop.is_set():
                try:
                    out = subprocess.run(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits"], capture_output=True, text=True,
                                         timeout=5).stdout.strip()
                    if out:
                        self.samples.append([x.strip() for x in out.split(",")])
                except Exception:
                    pass
                self._stop.wait(0.2)
        self._t = threading.Thread(target=run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *exc):
        self._stop.set()
        if self._t:
            self._t.join(timeout=6)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for s in self.samples for k in range(4) if len(s) > 3 + k and
                          s[3 + k].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            p = json.load(fh)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profiled_traffic_per_agent():
    """dram bytes per agent of k_agent from the committed ncu summary, if any."""
    p = os.path.join(ROOT, "profiles", "k_agent_socialforces_toric.md")
    try:
        for line in open(p):
            if line.startswith("traffic_bytes_per_agent:"):
                return float(line.split(":")[1])
    except OSError:
        pass
    return None


def cpu_baseline(path: str, n_agents: int, seconds: float = 12.0, threads: int | None = None):
    """The reference CPU step (compiled reference if present, else the CPU
    restatement) on all host cores, over a bounded number of steps."""
    threads = threads or os.cpu_count() or 1
    from oracle import ref as oref
    if oref.available():
        sim = oref.RefSim(path, threads=threads)
        kind = "reference"
    else:
        from oracle.port import PortSim
        sim = PortSim(path, threads=threads)
        kind = "port"
    t1 = sim.step(1)
    steps = max(1, min(200, int(seconds / max(t1, 1e-6))))
    t = sim.step(steps)
    return dict(value=n_agents * steps / t, unit="agent-steps/s", cores=threads, kind=kind,
                sample=f"{steps} steps of the full {n_agents}-agent workload after 1 warm-up step")


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
        return rank, world, local, dist
    return rank, world, local, None


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, x: float) -> float:
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_reference(args):
    rank, world, local, dist = dist_setup(args)
    if rank != 0:
        return
    with tempfile.TemporaryDirectory() as tmp:
        path, n, cfg = workload(args.workload, tmp)
        threads = os.cpu_count() or 1
        from oracle import ref as oref
        if oref.available():
            sim, kind = oref.RefSim(path, threads=threads), "reference"
        else:
            from oracle.port import PortSim
            sim, kind = PortSim(path, threads=threads), "port"
        sim.step(args.warmup)
        t = sim.step(args.steps)
        value = n * args.steps / t
        line = {"metric": METRIC, "impl": "reference", "value": value, "unit": "agent-steps/s",
                "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": 1e3 * t / args.steps, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)", "config": cfg,
                "cpu_baseline": {"value": value, "unit": "agent-steps/s", "cores": threads, "kind": kind,
                                 "sample": f"{args.steps} steps of the full workload after {args.warmup} warm-up"},
                "e2e": {"value": value, "unit": "agent-steps/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}}
        print(json.dumps(line))


def run_ours(args):
    rank, world, local, dist = dist_setup(args)
    from umans_gb300 import Simulation, UMANS
    from umans_gb300 import _lib
    import torch
    torch.cuda.set_device(local)
    with tempfile.TemporaryDirectory() as tmp:
        path, n, cfg = workload(args.workload, tmp)
        sim = Simulation(path)
        stream = torch.cuda.ExternalStream(sim.stream)
        flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")
        sim.step(args.warmup)
        # --- device-resident throughput, L2 flushed before every step ----
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
               for _ in range(args.steps)]
        torch.cuda.synchronize()
        barrier(dist)
        with ClockSampler(local) as clk:
            for k in range(args.steps):
                with torch.cuda.stream(stream):
                    flush.fill_(k & 0xff)
                    evs[k][0].record(stream)
                sim.step_async(1)
                evs[k][1].record(stream)
            sim.synchronize()
            torch.cuda.synchronize()
        barrier(dist)
        t_ms = sum(a.elapsed_time(b) for a, b in evs)
        t_ms = max_over_ranks(dist, t_ms)
        value = world * n * args.steps / (t_ms / 1e3)
        # --- back-to-back steps (L2 warm), for reference ------------------
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        sim.step_async(args.steps)
        t1.record(stream)
        sim.synchronize()
        warm_ms = t0.elapsed_time(t1)
        # --- dominant kernel: k_agent, CUDA events on the engine's stream --
        sim.profile(True)
        sim.step(max(10, min(args.steps, 50)))
        prof = sim.profile_totals()
        sim.profile(False)
        agent_ms = prof["agent_kernel_ms"] / max(prof["steps"], 1)
        step_ms_prof = prof["step_ms"] / max(prof["steps"], 1)
        ids, d2, cnt = sim.neighbours(cap=1)
        kbar = float(cnt.mean()) if n else 0.0
        peak, peak_kind = measured_peaks()
        alg_bytes = K_AGENT_BYTES_PER_AGENT * n
        achieved = alg_bytes / (agent_ms * 1e-3) / 1e9
        tpa = profiled_traffic_per_agent()
        flops = (SF_FLOP_PER_PAIR * kbar + SF_FLOP_PER_AGENT) * n
        clocks = clk.summary()
        sm_max = clocks.get("sm_max_mhz") or 2070.0
        fp32_peak = 152 * 128 * 2 * sm_max * 1e6 / 1e12
        sim.close()
        # --- e2e through the reference-facing C functions ----------------
        u = UMANS()
        assert u.startSimulation(path, 1)
        lib = _lib.load()
        ptr = C.POINTER(_lib.AgentData)()
        cnt_c = C.c_int()
        lib.GetAgentPositions(C.byref(ptr), C.byref(cnt_c))
        host = (_lib.AgentData * n)()
        C.memmove(host, ptr, C.sizeof(_lib.AgentData) * n)
        for _ in range(args.warmup):
            lib.SetAgentPositions(host, n)
            lib.DoSimulationSteps(1)
            lib.GetAgentPositions(C.byref(ptr), C.byref(cnt_c))
        barrier(dist)
        te = time.perf_counter()
        for _ in range(args.steps):
            lib.SetAgentPositions(host, n)
            lib.DoSimulationSteps(1)
            lib.GetAgentPositions(C.byref(ptr), C.byref(cnt_c))
            C.memmove(host, ptr, C.sizeof(_lib.AgentData) * n)
        te = time.perf_counter() - te
        te = max_over_ranks(dist, te)
        u.cleanUp()
        e2e_value = world * n * args.steps / te
        cpu = cpu_baseline(path, n) if (rank == 0 and world == 1 and not args.no_cpu) else None
    if rank != 0:
        return
    cfg = dict(cfg, l2="flushed (256 MiB write) before every timed step; state ~10 MB would fit in L2",
               neighbours_mean=round(kbar, 2), parallelism=f"replicas x{world}")
    line = {
        "metric": METRIC, "value": value, "unit": "agent-steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)", "config": cfg,
        "value_l2_warm": world * n * args.steps / (warm_ms / 1e3),
        "e2e": {"value": e2e_value, "unit": "agent-steps/s", "h2d_bytes_per_step": 28 * n * world,
                "d2h_bytes_per_step": 28 * n * world,
                "path": "SetAgentPositions -> DoSimulationSteps(1) -> GetAgentPositions, host buffers"},
        "roofline": {"bound": "hbm", "kernel": "k_agent", "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak, "peak_source": peak_kind,
                     "traffic": (tpa * n if tpa else None), "alg_bytes_per_launch": alg_bytes,
                     "launch_ms": agent_ms, "step_ms_profiled": step_ms_prof},
        "fp32_roofline": {"achieved_tflops": flops / (agent_ms * 1e-3) / 1e12, "peak_tflops_nominal": fp32_peak,
                          "frac": flops / (agent_ms * 1e-3) / 1e12 / fp32_peak,
                          "flop_per_agent_step": flops / max(n, 1)},
        "clocks": clocks,
        "gpu_launches": prof["kernels_per_step"] * args.steps,
    }
    if cpu:
        line["cpu_baseline"] = cpu
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="socialforces_toric")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
