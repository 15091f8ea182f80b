"""Times the compiled reference (oracle/_ref, built from the reference's own
sources by oracle/build_ref.sh) and the C restatement (oracle/port) on the
same scenario file, the same step range and the same thread counts, and
checks that they end in the same state.  Test infrastructure: it measures
how fast the oracle used as the CPU baseline on machines without the
reference's sources runs relative to the reference itself.

    UMANS_REFERENCE=<reference checkout> oracle/build_ref.sh
    python oracle/time_port_vs_ref.py [--agents N] [--warmup W] [--steps K]

Prints a summary and one line `port_over_reference: {json}`.
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--agents", type=int, default=100_000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--steps", type=int, default=20)
    args = ap.parse_args()
    from oracle import ref
    from oracle.port import PortSim
    from umans_gb300 import scenarios as S
    if not ref.available():
        raise SystemExit("oracle/_ref is not built (set UMANS_REFERENCE and run oracle/build_ref.sh)")
    cores = os.cpu_count() or 1
    rows = []
    with tempfile.TemporaryDirectory() as d:
        sc = S.socialforces_toric() if args.agents == 100_000 else \
            S.socialforces_toric(args.agents, density=100_000 / 400.0 ** 2)
        path = sc.write(os.path.join(d, "w.xml"))
        for threads in sorted({1, cores}):
            r = ref.RefSim(path, threads=threads)
            p = PortSim(path, threads=threads)
            r.step(args.warmup)
            p.step(args.warmup)
            tr = r.step(args.steps)
            tp = p.step(args.steps)
            same = bool(np.array_equal(r.state()["pos"], p.state()["pos"]))
            rows.append(dict(threads=threads, reference_s=tr, port_s=tp,
                             reference_agent_steps_per_s=args.agents * args.steps / tr,
                             port_agent_steps_per_s=args.agents * args.steps / tp,
                             port_over_reference=tr / tp, same_final_positions=same))
            r.close()
            p.close()
    for row in rows:
        print(f"threads {row['threads']:3d}: reference {row['reference_agent_steps_per_s']:.4g} agent-steps/s, "
              f"port {row['port_agent_steps_per_s']:.4g}, port/reference {row['port_over_reference']:.3g}, "
              f"same final positions {row['same_final_positions']}")
    out = {"value": rows[-1]["port_over_reference"], "threads": rows[-1]["threads"],
           "single_thread": rows[0]["port_over_reference"],
           "workload": f"SocialForces toric, {args.agents} agents, steps {args.warmup + 1}..{args.warmup + args.steps}",
           "rows": rows}
    print("port_over_reference: " + json.dumps(out))


if __name__ == "__main__":
    main()
