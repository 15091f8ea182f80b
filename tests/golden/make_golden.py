"""Generates the golden fixtures under tests/golden/ by running the UMANS
reference engine, compiled from its own sources (oracle/build_ref.sh), on
seeded scenarios from umans_gb300.scenarios.

Each fixture is an .npz holding the scenario XML (utf-8 bytes), the agent
ids, and the reference's float32 positions and velocities after the listed
steps; some also hold the reference's neighbour lists (ids and
PhantomAgent::distSqr in the reference's order) for the lists used in given
steps.  The arrivals40_* fixtures (timed insertion and remove-at-goal) hold
per snapshot the ids in the reference's list order and their positions.
Run from the repository root:

    python tests/golden/make_golden.py            # every fixture
    python tests/golden/make_golden.py arrivals   # the arrivals40_* ones
    python tests/golden/make_golden.py blocks     # the (toric_)blocks60_* ones

It needs oracle/_ref/libumans_ref.so, i.e. the reference sources.
"""
from __future__ import annotations

import os
import platform
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import ref  # noqa: E402
from umans_gb300 import scenarios as S  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def run(name, scen, steps, every=1, nb_steps=(), nb_agents=None):
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, name + ".xml")
        scen.write(path)
        xml = open(path, "rb").read()
        sim = ref.RefSim(path, threads=4)
        snaps, pos = [], []
        last = None
        nb = {}
        ids = sim.state()["ids"]
        for s in range(1, steps + 1):
            sim.step(1)
            if s % every == 0 or s == 1:
                st = sim.state()
                snaps.append(s)
                pos.append(st["pos"])
                last = st
            if s in nb_steps:
                agents = range(sim.n) if nb_agents is None else range(min(nb_agents, sim.n))
                lid, ld2, off = [], [], [0]
                for i in agents:
                    a, b, _ = sim.neighbors(i)
                    lid.append(a.astype(np.int32)); ld2.append(b)
                    off.append(off[-1] + len(a))
                nb[f"nb{s}_ids"] = np.concatenate(lid) if lid else np.zeros(0, np.int32)
                nb[f"nb{s}_d2"] = np.concatenate(ld2) if ld2 else np.zeros(0, np.float32)
                nb[f"nb{s}_off"] = np.array(off, np.int64)
        sim.close()
    np.savez_compressed(os.path.join(OUT, name + ".npz"), xml=np.frombuffer(xml, np.uint8),
                        ids=ids.astype(np.int32), steps=np.array(snaps, np.int32),
                        pos=np.array(pos, np.float32), vel_last=last["vel"], viewdir_last=last["viewdir"],
                        **nb)
    print(f"{name}: n={len(ids)} steps={steps} snapshots={len(snaps)}")


def run_dynamic(name, scen, steps, every=1):
    """Like run() for a changing population: each snapshot holds the ids in
    the reference's list order and their positions (ragged: snap_off)."""
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, name + ".xml")
        scen.write(path)
        xml = open(path, "rb").read()
        sim = ref.RefSim(path, threads=4)
        snaps, ids, pos, off = [], [], [], [0]
        for s in range(1, steps + 1):
            sim.step(1)
            if s % every == 0 or s == 1:
                st = sim.state()
                snaps.append(s)
                ids.append(st["ids"].astype(np.int32))
                pos.append(st["pos"].astype(np.float32))
                off.append(off[-1] + len(st["ids"]))
        sim.close()
    np.savez_compressed(os.path.join(OUT, name + ".npz"), xml=np.frombuffer(xml, np.uint8), dyn=np.int32(1),
                        steps=np.array(snaps, np.int32), snap_off=np.array(off, np.int64),
                        snap_ids=np.concatenate(ids), snap_pos=np.concatenate(pos).reshape(-1, 2))
    print(f"{name}: steps={steps} snapshots={len(snaps)} agents per snapshot {[len(i) for i in ids][:8]}...")


BLOCK_MODELS = ("SocialForces", "Karamouzas", "RVO", "Moussaid", "VanToll", "PLEdestrians", "PowerLaw")


def blocks():
    """Scenarios with hundreds of obstacle edges (the engine's edge grid)."""
    for m in BLOCK_MODELS:
        run(f"blocks60_{m}", S.model_block_field(m), 100, every=5)
    for m in ("SocialForces", "Karamouzas", "RVO"):
        run(f"toric_blocks60_{m}", S.model_toric_block_field(m), 100, every=5)


def main(only=None):
    if not ref.available():
        subprocess.check_call([os.path.join(ROOT, "oracle", "build_ref.sh")])
    if only == "arrivals":
        for m in S.MODEL_POLICIES:
            run_dynamic(f"arrivals40_{m}", S.model_arrivals(m), 100, every=5)
        return
    if only == "blocks":
        blocks()
        return
    for m in S.MODEL_POLICIES:
        run(f"circle24_{m}", S.model_circle(m), 100, every=5)
        run(f"crossing40_{m}", S.model_crossing(m), 100, every=5)
        run(f"toric60_{m}", S.model_toric(m, side=8.0), 100, every=5, nb_steps=(1,))
    for m in S.MODEL_POLICIES:
        run(f"obstacle_crossing40_{m}", S.model_obstacle_crossing(m), 100, every=5)
        run(f"corridor_walls40_{m}", S.model_corridor_walls(m), 100, every=5)
        run(f"toric_obstacle60_{m}", S.model_toric_obstacle(m), 100, every=5)
    for name in S.REGISTRY_POLICIES:
        run(f"registry40_{name}", S.registry_crossing(name), 100, every=5)
    run("orca_circle50", S.circle_orca(50), 100, every=5, nb_steps=(1, 50))
    run("socialforces_toric1500", S.socialforces_toric(n=1500, density=0.625), 100, every=10,
        nb_steps=(1, 100), nb_agents=150)
    run("karamouzas_corridor1200", S.karamouzas_corridor(n=1200, width=20.0), 40, every=10,
        nb_steps=(1,), nb_agents=60)
    for k, n in ((0, 40), (1, 90), (2, 150), (3, 64), (4, 120), (5, 33)):
        run(f"batch{k}_n{n}", S.batch_member(k, n), 60, every=5)
    run("calibration512", S.calibration_set(), 100, every=10)
    for m in S.MODEL_POLICIES:
        run_dynamic(f"arrivals40_{m}", S.model_arrivals(m), 100, every=5)
    blocks()
    with open(os.path.join(OUT, "PROVENANCE.txt"), "w") as fh:
        cc = subprocess.run(["g++", "--version"], capture_output=True, text=True).stdout.splitlines()[0]
        fh.write("Golden fixtures: UMANS reference engine compiled from its own sources by\n"
                 "oracle/build_ref.sh (g++ -O2 -std=c++17 -fopenmp -ffp-contract=off),\n"
                 f"compiler: {cc}\nhost: {platform.machine()} {platform.system()}\n"
                 "generator: tests/golden/make_golden.py (scenarios from umans_gb300/scenarios.py)\n")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else None)
