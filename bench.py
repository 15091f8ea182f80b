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
import contextlib
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
# algorithmic bytes of the grid build (k_count, k_scan_*, k_scatter) per agent:
# k_count reads scenario 4 + pos 8, writes cell 4                  = 16 B
# k_scatter reads cell 4, pos 8, goal 8, parameters 16, vel 8, id 4,
#           writes pref 8, sP 8, sV 8, sB 16, sE 16, slot 4, id 4  = 112 B
# (the per-cell histogram and scan, 16 B per cell, are not counted: ~4 B per
# agent on the 100k-agent toric workload's 160 x 160 cells)
GRID_BYTES_PER_AGENT = 128
# FP32 operations per neighbour pair, counted from the reference source
# (SocialForcesAvoidance.cpp:26-110 ~55, contact term policy.cpp:107-141 ~12),
# plus ~40 per agent (goal force, clamps, integration)
SF_FLOP_PER_PAIR = 67
SF_FLOP_PER_AGENT = 40
# FP32 operations of one pair collision time (costFunction.cpp:173-227: the
# quadratic with one sqrt and two divisions, the range and zero tests)
KARAMOUZAS_FLOP_PER_TTC = 30


def workload(name: str, tmp: str, agents: int = 0):
    """agents > 0 scales the SocialForces workload at the same density
    (smaller cases for profiler captures)."""
    from umans_gb300 import scenarios as S
    if name == "socialforces_toric":
        n = agents or 100_000
        sc = S.socialforces_toric(n, density=100_000 / 400.0 ** 2) if agents else S.socialforces_toric()
        side = math.sqrt(n / (100_000 / 400.0 ** 2))
        cfg = dict(workload="socialforces_toric", agents=n, world=f"toric {side:.0f}x{side:.0f} m",
                   policy="SocialForcesAvoidance(range 5)+GoalReachingForce, gradient", dt=0.1)
    elif name == "karamouzas_corridor":
        n = agents or 1_000_000
        sc = S.karamouzas_corridor(n)
        cfg = dict(workload="karamouzas_corridor", agents=n, world=f"infinite, {n // 100}x100 m corridor",
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


def fp32_peak_tflops(sm_mhz: float) -> tuple[float, int]:
    """Nominal FP32 peak of the device: SMs (read from the device) x 128 FP32
    lanes x 2 FLOP (FMA) x the SM clock.  MEASURED_PEAKS.json holds no FP32
    figure, so this is the denominator of the FP32 roofline."""
    import torch
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    return sms * 128 * 2 * sm_mhz * 1e6 / 1e12, sms


def port_over_reference():
    """Speed of the C restatement relative to the compiled reference on the
    same workload, from the committed CPU measurement (profiles/), if any."""
    p = os.path.join(ROOT, "profiles", "cpu_port_vs_reference.md")
    try:
        for line in open(p):
            if line.startswith("port_over_reference:"):
                return json.loads(line.split(":", 1)[1])
    except (OSError, ValueError):
        pass
    return None


def profiled_traffic_per_agent():
    """dram bytes per agent of k_force_quad from the committed ncu summary, if any."""
    p = os.path.join(ROOT, "profiles", "k_force_quad_socialforces_toric.md")
    try:
        for line in open(p):
            if line.startswith("traffic_bytes_per_agent:"):
                return float(line.split(":")[1])
    except OSError:
        pass
    return None


def batched_leg(tmp: str, steps: int, warmup: int, flush, stream_of):
    """4096 independent scenarios (agent counts log-uniform in [8, 2048],
    circle / random-square layouts, ORCA / PowerLaw-sampling / SocialForces)
    stepped together, against the plain path run scenario by scenario."""
    import torch
    from umans_gb300 import Batch, Simulation, scenarios as S
    counts = S.batch_counts()
    paths = [S.batch_member(k, int(n)).write(os.path.join(tmp, f"batch_{k}.xml")) for k, n in enumerate(counts)]
    total = int(counts.sum())
    b = Batch(paths)
    b.step(warmup)
    tune = b.autotune(trial_steps=2)
    st = torch.cuda.ExternalStream(b.stream)
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    torch.cuda.synchronize()
    for k in range(steps):
        with torch.cuda.stream(st):
            flush.fill_(k & 0xff)
            evs[k][0].record(st)
        b.step_async(1)
        evs[k][1].record(st)
    b.synchronize()
    torch.cuda.synchronize()
    t_ms = sum(a.elapsed_time(c) for a, c in evs)
    batched = total * steps / (t_ms / 1e3)
    b.close()
    # plain path, one scenario after another (every 16th scenario), timed
    # with CUDA events on each simulation's stream like the batch (its steps
    # are enqueued back to back; the flush of the batch timing is left out,
    # which favours the plain path)
    sample = list(range(0, len(paths), 16))
    plain_agent_steps, plain_ms = 0, 0.0
    psteps = 10
    for k in sample:
        sim = Simulation(paths[k])
        sim.step(2)
        pst = torch.cuda.ExternalStream(sim.stream)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(pst)
        sim.step_async(psteps)
        e1.record(pst)
        sim.synchronize()
        plain_ms += e0.elapsed_time(e1)
        plain_agent_steps += int(counts[k]) * psteps
        sim.close()
    plain = plain_agent_steps / (plain_ms / 1e3)
    return {"value": batched, "unit": "agent-steps/s", "scenarios": len(paths), "agents": total, "steps": steps,
            "ms_per_step": t_ms / steps, "autotune": tune,
            "plain_per_scenario": {"value": plain, "unit": "agent-steps/s",
                                   "sample": f"{len(sample)} of {len(paths)} scenarios (every 16th), {psteps} steps each, "
                                             "one Simulation per scenario, sequentially",
                                   "timing": "CUDA events on each simulation's stream, the same clock as the batch"},
            "speedup_vs_plain": batched / plain}


def diff_leg(tmp: str, sets: int = 256, n: int = 512, steps: int = 100, every: int = 10, reps: int = 3):
    """Differentiable form: `sets` parameter sets (V0, sigma, k, tau0 within
    +-30% of the defaults) x `n` agents (random 40 x 40 m square, seeded
    goals), one batch; loss = mean squared position error over `steps`
    steps against the trajectories of a held-out parameter set; checkpoint
    every `every` steps.  Times the forward episode, the adjoint (recompute
    + reverse), and plain stepping of the same batch."""
    import torch
    from umans_gb300 import Batch, Simulation, scenarios as S
    params = S.calibration_params(sets)
    held = S.calibration_set((2.52, 0.255, 1.65, 2.7), n=n).write(os.path.join(tmp, "held.xml"))
    h = Simulation(held)
    tg = np.empty((steps, n, 2), np.float32)
    obs = {"pos": [], "vel": [], "viewdir": []}
    for t in range(steps + 1):
        st = h.state()
        for k in obs:
            obs[k].append(st[k].copy())
        if t < steps:
            h.step(1)
            tg[t] = h.positions()
    h.close()
    paths = [S.calibration_set(params[k], n=n).write(os.path.join(tmp, f"cal_{k}.xml")) for k in range(sets)]
    b = Batch(paths)
    targets = np.ascontiguousarray(np.tile(tg, (1, sets, 1)))
    b.diff_begin(targets, checkpoint_every=every)
    fwd, bwd, plain = [], [], []
    for r in range(reps + 1):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        loss = b.diff_forward()
        t1 = time.perf_counter()
        g = b.diff_backward()
        t2 = time.perf_counter()
        if r:
            fwd.append(t1 - t0)
            bwd.append(t2 - t1)
    start = b.state()   # diff_backward leaves the episode's start state
    for r in range(reps + 1):
        b.set_state(start["pos"], start["vel"], start["viewdir"])
        b.synchronize()
        t0 = time.perf_counter()
        b.step(steps)
        b.synchronize()
        if r:
            plain.append(time.perf_counter() - t0)
    # windowed calibration (multiple shooting): windows of `every` steps, each
    # from the observed state at its start
    from umans_gb300.calibration import windowed_gradient
    tiled = {k: np.ascontiguousarray(np.tile(np.array(v, np.float32), (1, sets, 1))) for k, v in obs.items()}
    b.synchronize()
    t0 = time.perf_counter()
    wloss, wg = windowed_gradient(b, tiled, window=every)
    wsec = time.perf_counter() - t0
    params_eng = [b.force_params(k).astype(np.float64) for k in range(sets)]
    b.close()
    # the first window's gradient of a sample of sets against the float64
    # tangent along their own trajectories (oracle/calib64.py)
    check = None
    try:
        from oracle import calib64, port as oport
        sample = [k for k in (0, sets // 4, sets // 2, 3 * sets // 4) if k < sets]
        b1 = Batch([paths[k] for k in sample])
        t1 = {k: np.ascontiguousarray(np.tile(np.array(v[:every + 1], np.float32), (1, len(sample), 1)))
              for k, v in obs.items()}
        for j, k in enumerate(sample):
            b1.set_force_params(params_eng[k].astype(np.float32), j)
        _, g1 = windowed_gradient(b1, t1, window=every)
        b1.close()
        errs, engs, refs = [], [], []
        z = np.zeros((n, 2))
        for j, k in enumerate(sample):
            s = Simulation(paths[k])
            st = []
            for tt in range(every + 1):
                x = s.state()
                st.append((x["pos"].copy(), x["vel"].copy()))
                if tt < every:
                    s.step(1)
            s.close()
            ref = calib64.tangent_gradient(oport.read_scenario(paths[k]), st, np.array(obs["pos"][1:every + 1]),
                                           1.0 / (every * n), params_eng[k], [(np.eye(4)[q], z, z) for q in range(4)],
                                           h=1e-8)
            errs.append(float(np.linalg.norm(g1[j] - ref) / max(np.linalg.norm(ref), 1e-30)))
            engs.append(np.asarray(g1[j], np.float64))
            refs.append(ref)
        e_all, r_all = np.concatenate(engs), np.concatenate(refs)
        check = {"sets": sample, "window": f"steps 1..{every}",
                 "rel_err_vs_float64_tangent": float(np.linalg.norm(e_all - r_all) / max(np.linalg.norm(r_all), 1e-30)),
                 "per_set": errs, "tolerance": 1e-3,
                 "metric": "2-norm over the sampled sets' 4 parameters each, as the tests"}
    except Exception as e:   # the check is a report, not part of the timing
        check = {"error": repr(e)}
    finite = np.isfinite(g).all(1)
    f, a, p = statistics.median(fwd), statistics.median(bwd), statistics.median(plain)
    return {"sets": sets, "agents_per_set": n, "steps": steps, "checkpoint_every": every,
            "forward_episode_s": f, "adjoint_s": a, "plain_steps_s": p,
            "forward_ms_per_step": 1e3 * f / steps, "fwd_adjoint_ms_per_step": 1e3 * (f + a) / steps,
            "fwd_adjoint_over_forward": (f + a) / f, "fwd_adjoint_over_plain_step": (f + a) / p,
            "agent_steps_per_s_forward": sets * n * steps / f,
            "loss": loss, "sets_with_finite_gradient": int(finite.sum()),
            "gradient_note": "over 100 steps at this density the pathwise gradient of one episode grows ~2.5x "
                             "per step (the forward map's own divergence rate) and leaves the float range; "
                             "the windowed form below is the one to calibrate with",
            "windowed": {"windows": (steps + every - 1) // every, "window_steps": every, "seconds": wsec,
                         "ms_per_step": 1e3 * wsec / steps, "loss": wloss,
                         "sets_with_finite_gradient": int(np.isfinite(wg).all(1).sum()),
                         "gradient_check": check},
            "timing": f"median of {reps} after one warm-up, host clock around synchronous calls; "
                      "inputs (tape ~0.7 GB) exceed L2"}


def config_leg(name: str, tmp: str, steps: int, warmup: int, flush, cpu_agents: int = 0,
               cpu_seconds: float = 10.0, whole_run: bool = False) -> dict:
    """Another configuration of the reference's benchmark list, timed like the
    headline (per-step CUDA events, L2 flushed before each step), with the
    reference CPU step beside it (on the full case, or on a smaller case at
    the same density when the full one would take minutes per step).

    whole_run: the configuration's whole run (`steps` steps from the initial
    state) is also timed as one call, the way the reference's
    RunSimulationSteps runs it; small worlds then step inside one launch.
    That figure becomes the leg's value, the per-step one is kept beside it."""
    import torch
    from umans_gb300 import Simulation
    sub = os.path.join(tmp, name)
    os.makedirs(sub, exist_ok=True)
    t0 = time.perf_counter()
    path, n, cfg = workload(name, sub)
    t_write = time.perf_counter() - t0
    sim = Simulation(path)
    t_load = time.perf_counter() - t0 - t_write
    stream = torch.cuda.ExternalStream(sim.stream)
    sim.step(warmup)
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    torch.cuda.synchronize()
    for k in range(steps):
        with torch.cuda.stream(stream):
            flush.fill_(k & 0xff)
            evs[k][0].record(stream)
        sim.step_async(1)
        evs[k][1].record(stream)
    sim.synchronize()
    torch.cuda.synchronize()
    t_ms = sum(a.elapsed_time(b) for a, b in evs)
    work = None
    if name == "karamouzas_corridor":
        # samples inside the Karamouzas window and pair collision times, counted
        # in the kernel over two profiled steps (FLOPs as counted from the
        # reference source: ~30 per pair collision time, the preferred-velocity
        # sweep once per agent plus one sweep per window sample)
        sim.profile(True)
        sim.step(2)
        pr = sim.profile_totals()
        cn = sim.profile_counters()
        sim.profile(False)
        agents = max(cn["karamouzas_agents"], 1)
        s_eval = cn["karamouzas_window_samples"] / agents
        kbar = cn["karamouzas_pair_ttc"] / max(cn["karamouzas_window_samples"], 1)
        flop = KARAMOUZAS_FLOP_PER_TTC * kbar * (1.0 + s_eval)
        kms = pr["agent_kernel_ms"] / max(pr["steps"], 1)
        fp32_peak, sms = fp32_peak_tflops(2070.0)
        work = dict(sms=sms, window_samples_per_agent=s_eval, pairs_per_sample=kbar, flop_per_agent_step=flop,
                    k_agent_ms=kms, achieved_tflops=flop * n / (kms * 1e-3) / 1e12,
                    peak_tflops_nominal=fp32_peak, frac=flop * n / (kms * 1e-3) / 1e12 / fp32_peak)
    sim.close()
    out = dict(config=dict(cfg, timed_steps=f"steps {warmup + 1}..{warmup + steps}",
                           l2="flushed (256 MiB write) before every timed step"),
               value=n * steps / (t_ms / 1e3), unit="agent-steps/s", steps=steps, warmup=warmup,
               ms_per_step=t_ms / steps)
    if whole_run:
        runs = []
        for k in range(warmup + 1):   # the first runs warm up, the last is timed
            sim = Simulation(path)
            stream = torch.cuda.ExternalStream(sim.stream)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            with torch.cuda.stream(stream):
                flush.fill_(k & 0xff)
                e0.record(stream)
            sim.step_async(steps)
            e1.record(stream)
            sim.synchronize()
            torch.cuda.synchronize()
            runs.append(e0.elapsed_time(e1))
            launches = sim.profile_totals()["kernels_per_step"]
            sim.close()
        w_ms = runs[-1]
        out["one_step_per_call"] = dict(value=out["value"], ms_per_step=out["ms_per_step"],
                                        timed_steps=out["config"]["timed_steps"])
        out["value"] = n * steps / (w_ms / 1e3)
        out["ms_per_step"] = w_ms / steps
        out["config"]["timed_steps"] = f"the whole run, steps 1..{steps}, as one call ({warmup} untimed runs before)"
        out["config"]["l2"] = "flushed (256 MiB write) before the timed run"
        out["whole_run"] = dict(ms=w_ms, launches_per_call=launches if launches == 1 else launches * steps)
    if work:
        out["fp32_roofline"] = work
    t_gpu = time.perf_counter() - t0 - t_write - t_load
    if cpu_agents >= 0:
        cpath, cn = path, n
        if cpu_agents:
            csub = os.path.join(sub, "cpu")
            os.makedirs(csub, exist_ok=True)
            cpath, cn, _ = workload(name, csub, cpu_agents)
        cb = cpu_baseline(cpath, cn, seconds=cpu_seconds, max_steps=steps if not cpu_agents else 10_000)
        if cpu_agents:
            cb["sample"] = cb["sample"].replace("full", "same-density") + f" (the GPU case has {n} agents)"
        out["cpu_baseline"] = cb
    out["leg_seconds"] = dict(write_scenario=round(t_write, 1), load=round(t_load, 1), gpu=round(t_gpu, 1),
                              cpu=round(time.perf_counter() - t0 - t_write - t_load - t_gpu, 1))
    return out


def cpu_baseline(path: str, n_agents: int, seconds: float = 30.0, threads: int | None = None, max_steps: int = 500):
    """The reference CPU step (compiled reference if present, else the CPU
    restatement) on all host cores, over a bounded number of steps."""
    threads = threads or os.cpu_count() or 1
    from oracle import ref as oref
    with native_stdout_to_stderr():
        if oref.available():
            sim = oref.RefSim(path, threads=threads)
            kind = "reference"
        else:
            from oracle.port import PortSim
            sim = PortSim(path, threads=threads)
            kind = "port"
        t1 = sim.step(1)
        # the per-step cost grows as the crowd condenses: time the same step
        # range as the GPU when the budget allows
        steps = max(1, min(max_steps, int(seconds / max(t1, 1e-6) / 1.3)))
        t = sim.step(steps)
    return dict(value=n_agents * steps / t, unit="agent-steps/s", cores=threads, kind=kind,
                sample=f"{steps} steps of the full {n_agents}-agent workload after 1 warm-up step")


def parity_leg(path: str, warmup: int, steps: int, threads: int | None = None, checks: int = 5) -> dict:
    """Maximum per-agent position deviation of the GPU trajectory from the
    oracle (the C restatement, pinned to the reference by the golden
    fixtures) over the benchmark's own step range, compared `checks` times."""
    from oracle.port import PortSim
    from umans_gb300 import Simulation
    threads = threads or os.cpu_count() or 1
    sim = Simulation(path)
    with native_stdout_to_stderr():
        port = PortSim(path, threads=threads)
    sim.step(warmup)
    port.step(warmup)
    done, dev, worst_step = warmup, 0.0, warmup
    left = steps
    while left > 0:
        k = min(left, max(1, steps // checks))
        sim.step(k)
        port.step(k)
        done += k
        left -= k
        d = float(np.abs(sim.positions() - port.state()["pos"]).max())
        if d > dev:
            dev, worst_step = d, done
    sim.close()
    port.close()
    return {"max_dev_m": dev, "at_step": worst_step, "steps_compared": f"{warmup + 1}..{done}",
            "against": "oracle (C restatement, bit-identical to the compiled reference on the golden fixtures)",
            "bar_m": 1e-4}


def dist_setup(args=None, backend: str | None = None):
    """One process per GPU under torchrun: every rank runs an independent
    replica of the workload (the step has no exchange between replicas);
    the process group only carries the barrier and the max over ranks.
    NCCL on GPUs; gloo where there is no GPU (the CPU tests)."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        if backend is None:
            backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
        return rank, world, local, dist
    return rank, world, local, None


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, x: float) -> float:
    if dist is None:
        return x
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_rate(world: int, agents: int, steps: int, seconds: float) -> float:
    """Whole-job agent-steps/s of `world` replicas of `agents` agents that
    all finished `steps` steps within `seconds` (the slowest rank's time)."""
    return world * agents * steps / seconds


@contextlib.contextmanager
def native_stdout_to_stderr():
    """Sends what native code writes to standard output (the reference engine
    reports world creation there) to standard error, so that standard output
    carries the JSON line alone."""
    libc = C.CDLL(None)
    sys.stdout.flush()
    saved = os.dup(1)
    os.dup2(2, 1)
    try:
        yield
    finally:
        libc.fflush(None)
        sys.stdout.flush()
        os.dup2(saved, 1)
        os.close(saved)


def run_reference(args):
    rank, world, local, dist = dist_setup(args)
    if rank != 0:
        return
    with tempfile.TemporaryDirectory() as tmp, native_stdout_to_stderr():
        path, n, cfg = workload(args.workload, tmp, args.agents)
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
    por = port_over_reference()
    if kind == "port" and por is not None:
        line["cpu_baseline"]["port_over_reference"] = por
    print(json.dumps(line))


def run_ours(args):
    rank, world, local, dist = dist_setup(args)
    from umans_gb300 import Simulation, UMANS
    from umans_gb300 import _lib
    import torch
    torch.cuda.set_device(local)
    with tempfile.TemporaryDirectory() as tmp:
        if args.only_leg:
            # one leg alone (a short command for profiling its kernels)
            if args.only_leg == "batched":
                flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")
                out = batched_leg(tmp, min(args.steps, 20), args.warmup, flush, None)
            else:
                out = diff_leg(tmp, sets=args.diff_sets)
            if rank == 0:
                print(json.dumps({"leg": args.only_leg, "result": out}))
            return
        legs = {}
        tl = time.perf_counter()

        def lap(name):
            nonlocal tl
            now = time.perf_counter()
            legs[name] = round(now - tl, 1)
            tl = now
        path, n, cfg = workload(args.workload, tmp, args.agents)
        sim = Simulation(path)
        stream = torch.cuda.ExternalStream(sim.stream)
        flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")
        lap("setup")
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
        value = replica_rate(world, n, args.steps, t_ms / 1e3)
        sim.close()
        lap("plain")
        # --- back-to-back steps (L2 warm), same step range, fresh state ----
        sim = Simulation(path)
        stream = torch.cuda.ExternalStream(sim.stream)
        sim.step(args.warmup)
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        sim.step_async(args.steps)
        t1.record(stream)
        sim.synchronize()
        warm_ms = t0.elapsed_time(t1)
        sim.close()
        # --- dominant kernel: k_force_quad, CUDA events on the engine's stream,
        # over the same step range (fresh state); mean neighbour count sampled
        sim = Simulation(path)
        sim.step(args.warmup)
        sim.profile(True)
        kb, left = [], args.steps
        while left > 0:
            k = min(left, max(1, args.steps // 5))
            sim.step(k)
            left -= k
            kb.append(float(sim.neighbours(cap=1)[2].mean()) if n else 0.0)
        prof = sim.profile_totals()
        sim.profile(False)
        agent_ms = prof["agent_kernel_ms"] / max(prof["steps"], 1)
        step_ms_prof = prof["step_ms"] / max(prof["steps"], 1)
        grid_ms = prof["grid_build_ms"] / max(prof["steps"], 1)
        kbar = sum(kb) / len(kb)
        list_cap = sim.max_neighbours
        peak, peak_kind = measured_peaks()
        alg_bytes = K_AGENT_BYTES_PER_AGENT * n
        achieved = alg_bytes / (agent_ms * 1e-3) / 1e9
        tpa = profiled_traffic_per_agent()
        flops = (SF_FLOP_PER_PAIR * kbar + SF_FLOP_PER_AGENT) * n
        clocks = clk.summary()
        sm_max = clocks.get("sm_max_mhz") or 2070.0
        fp32_peak, sms = fp32_peak_tflops(sm_max)
        sim.close()
        lap("warm_and_profile")
        # --- e2e through the reference-facing C functions ----------------
        u = UMANS()
        assert u.startSimulation(path, 1)
        lib = _lib.load()
        ptr = C.POINTER(_lib.AgentData)()
        cnt_c = C.c_int()
        lib.GetAgentPositions(C.byref(ptr), C.byref(cnt_c))
        host = (_lib.AgentData * n)()
        C.memmove(host, ptr, C.sizeof(_lib.AgentData) * n)
        # each step sends the previous step's records back (the buffer
        # GetAgentPositions returned, a host buffer owned by the library)
        cur = host
        for _ in range(args.warmup):
            lib.SetAgentPositions(cur, n)
            lib.DoSimulationSteps(1)
            lib.GetAgentPositions(C.byref(ptr), C.byref(cnt_c))
            cur = ptr
        barrier(dist)
        te = time.perf_counter()
        for _ in range(args.steps):
            lib.SetAgentPositions(cur, n)
            lib.DoSimulationSteps(1)
            lib.GetAgentPositions(C.byref(ptr), C.byref(cnt_c))
            cur = ptr
        te = time.perf_counter() - te
        te = max_over_ranks(dist, te)
        u.cleanUp()
        e2e_value = replica_rate(world, n, args.steps, te)
        lap("e2e")
        cpu = cpu_baseline(path, n, max_steps=args.steps) if (rank == 0 and world == 1 and not args.no_cpu) else None
        if cpu is not None:
            por = port_over_reference()
            if por is not None:
                cpu["port_over_reference"] = por
        lap("cpu_baseline")
        parity = parity_leg(path, args.warmup, args.steps) if (rank == 0 and not args.no_parity) else None
        lap("parity")
        batched = None if args.no_batch else batched_leg(tmp, min(args.steps, 20), args.warmup, flush, None)
        lap("batched")
        diff = None if args.no_diff else diff_leg(tmp, sets=args.diff_sets)
        lap("differentiable")
        extra = None
        if not args.no_extra and world == 1:
            extra = {"small_orca_circle": config_leg("circle_orca", tmp, 300, args.warmup, flush,
                                                     cpu_agents=0 if not args.no_cpu else -1, whole_run=True),
                     "sampling_heavy_karamouzas": config_leg("karamouzas_corridor", tmp, 5, 3, flush,
                                                             cpu_agents=20_000 if not args.no_cpu else -1)}
        lap("other_configs")
    if rank != 0:
        return
    cfg = dict(cfg, l2="flushed (256 MiB write) before every timed step; state ~10 MB would fit in L2",
               timed_steps=f"steps {args.warmup + 1}..{args.warmup + args.steps} of the scenario (the neighbour "
                           f"count grows as the crowd condenses)",
               neighbours_mean=round(kbar, 2), list_capacity=list_cap, parallelism=f"replicas x{world}")
    line = {
        "metric": METRIC, "value": value, "unit": "agent-steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)", "config": cfg,
        "value_l2_warm": world * n * args.steps / (warm_ms / 1e3),
        "e2e": {"value": e2e_value, "unit": "agent-steps/s", "h2d_bytes_per_step": 28 * n * world,
                "d2h_bytes_per_step": 28 * n * world,
                "path": "SetAgentPositions -> DoSimulationSteps(1) -> GetAgentPositions, host buffers"},
        # the kernel's bound is min(HBM / bytes, FP32 / FLOPs) per agent-step;
        # with ~96 B and ~3.3 kFLOP per agent-step the FP32 term is the lower
        "roofline": {"bound": "fp32", "kernel": "k_force_quad",
                     "achieved": flops / (agent_ms * 1e-3) / 1e12, "peak": fp32_peak, "unit": "TFLOP/s",
                     "frac": flops / (agent_ms * 1e-3) / 1e12 / fp32_peak,
                     "peak_source": f"nominal: {sms} SMs (from the device) x 128 FP32 lanes x 2 FLOP x "
                                    f"{sm_max:.0f} MHz; MEASURED_PEAKS.json has no FP32 figure",
                     "flop_per_agent_step": flops / max(n, 1),
                     "flop_count": f"{SF_FLOP_PER_PAIR} per neighbour pair x {kbar:.1f} neighbours + "
                                   f"{SF_FLOP_PER_AGENT} per agent (counted from the reference source)",
                     "traffic": (tpa * n if tpa else None), "traffic_unit": "DRAM bytes per launch (ncu)",
                     "launch_ms": agent_ms, "step_ms_profiled": step_ms_prof,
                     "agent_steps_roofline": min(peak * 1e9 / K_AGENT_BYTES_PER_AGENT,
                                                 fp32_peak * 1e12 / (flops / max(n, 1))),
                     "frac_of_agent_steps_roofline": (n / (agent_ms * 1e-3)) /
                                                     min(peak * 1e9 / K_AGENT_BYTES_PER_AGENT,
                                                         fp32_peak * 1e12 / (flops / max(n, 1)))},
        "hbm_roofline": {"kernel": "k_force_quad", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_source": peak_kind, "alg_bytes_per_launch": alg_bytes,
                         "traffic": (tpa * n if tpa else None)},
        "grid_build": {"kernels": "k_count_scan, k_scatter (static toric grid)", "ms": grid_ms,
                       # null when the two legs' kernels differ (e.g. a capacity change in one leg)
                       "ms_in_graph": (t_ms / args.steps - agent_ms) if t_ms / args.steps > agent_ms else None,
                       "alg_bytes_per_agent": GRID_BYTES_PER_AGENT,
                       "achieved": GRID_BYTES_PER_AGENT * n / (grid_ms * 1e-3) / 1e9 if grid_ms > 0 else None,
                       "peak": peak, "unit": "GB/s",
                       "frac": GRID_BYTES_PER_AGENT * n / (grid_ms * 1e-3) / 1e9 / peak if grid_ms > 0 else None,
                       "note": "ms: profiled steps (separate launches, with their launch gaps); ms_in_graph: the "
                               "graph-replayed step minus the agent kernel (grid build and graph launch)"},
        "clocks": clocks,
        "gpu_launches": prof["kernels_per_step"] * args.steps,
    }
    if cpu:
        line["cpu_baseline"] = cpu
    if parity:
        line["max_dev_m"] = parity["max_dev_m"]
        line["parity"] = parity
    if batched:
        line["batched"] = batched
    if diff:
        line["differentiable"] = diff
    if extra:
        line["other_configs"] = extra
    line["leg_seconds"] = legs
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=500,
                    help="timed steps (default: the 500 steps of the plain large workload)")
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="socialforces_toric")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-parity", action="store_true", help="skip the deviation check against the oracle")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-form leg")
    ap.add_argument("--no-diff", action="store_true", help="skip the differentiable-form leg")
    ap.add_argument("--no-extra", action="store_true",
                    help="skip the small ORCA and sampling-heavy Karamouzas configurations")
    ap.add_argument("--agents", type=int, default=0,
                    help="agents of the SocialForces workload at the same density (default 100000)")
    ap.add_argument("--diff-sets", type=int, default=256, help="parameter sets of the differentiable leg")
    ap.add_argument("--only-leg", choices=["batched", "diff"], default=None,
                    help="run one leg alone and print its record (for profiling; not a bench line)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
