"""Count the FP64 work per segment of the reference's tracking algorithm on the
benchmark workloads (test infrastructure), with the C restatement's counters
(oracle/qs_oracle.c: every +, -, *, / and sqrt of a double as the reference
writes it, on the tracking path; log / sin / cos / exp calls apart).  Writes
``profiles/fp64_work_per_segment.json``, which bench.py reads for the FP64
FLOP roofline (the algorithm's operations per segment x the measured segment
rate against the GPU's measured FP64 rate) and tests/test_oracle_fp64_work.py
checks against a fresh count.

The algorithm evaluates all 24 facets of the cell on every segment
(MCT.cc:549-621); the library's FP32 screen skips most of them, so the GPU
executes far fewer FP64 operations than these counts -- the counts are the
work the reference's algorithm asks for, the GPU's own are in the ncu
profile.

Usage: python tests/golden/count_fp64_work.py
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))
sys.path.insert(0, str(ROOT / "tests"))

OUT = ROOT / "profiles" / "fp64_work_per_segment.json"

# workload -> (decks, cycles counted, particles per deck or None for the deck's own)
WORKLOADS = {
    "config1": "10^3 cells, 1 material, 1e5 particles, all 10 cycles",
    "config2": "40^3 cells, 3 materials, 1e6 particles, cycles 0-2",
    "config3": "the ensemble's first 16 problems, cycles 0-1 each",
    "config4": "10^3 cells, 3 materials, escape, 1e6 particles, cycles 0-2",
    "config5": "one replica (64^3 cells, 5 slabs) at 3e6 particles, cycles 0-1",
}


def count_run(hp, sim, cycles: int, seed_offset: int = 0) -> tuple[int, int, int]:
    """(segments, FP64 operations, elementary calls) of `cycles` whole cycles."""
    import oracle_py as O
    from helpers import oracle_run
    run = oracle_run(hp, sim)
    if seed_offset:
        run.set_seed_offset(seed_offset)
    segments = 0
    O.flop_counts(reset=True)
    for _ in range(cycles):
        run.cycle_init()
        run.cycle_tracking(0)
        run.cycle_finalize()
        segments += int(run.last_balance()[12])
    flops, elem = O.flop_counts(reset=True)
    run.close()
    return segments, flops, elem


def count_workload(name: str) -> dict:
    from quicksilver_gb300 import Deck
    from quicksilver_gb300.monte_carlo import seed_offset
    from helpers import load_problem
    totals = [0, 0, 0]
    if name in ("config1", "config2", "config4"):
        cycles = {"config1": 10, "config2": 3, "config4": 3}[name]
        _, sim, hp = load_problem(f"{name}.inp", {"nSteps": cycles})
        runs = [(hp, sim, cycles, 0)]
    elif name == "config3":
        from quicksilver_gb300.decks.make_decks import config3
        decks = [Deck.from_string(t, {"nSteps": 2}) for t in config3()[:16]]
        runs = [(d.build(), d.simulation, 2, seed_offset(d.simulation.seed)) for d in decks]
    else:
        from quicksilver_gb300.decks.make_decks import config5
        d = Deck.from_string(config5(n_particles=3_000_000)[0], {"nSteps": 2})
        runs = [(d.build(), d.simulation, 2, seed_offset(d.simulation.seed))]
    for hp, sim, cycles, off in runs:
        for k, v in enumerate(count_run(hp, sim, cycles, off)):
            totals[k] += v
    segments, flops, elem = totals
    return {"workload": WORKLOADS[name], "segments": segments, "fp64_ops": flops, "elementary_calls": elem,
            "fp64_ops_per_segment": round(flops / segments, 2),
            "elementary_calls_per_segment": round(elem / segments, 4)}


def main(argv: list[str]) -> None:
    names = argv or list(WORKLOADS)
    data = json.loads(OUT.read_text()) if OUT.exists() else {}
    data["rules"] = ("FP64 +, -, *, / and sqrt of the tracking path as the reference writes them "
                     "(multiplications by -1.0 included; comparisons, conversions and the macroscopic total "
                     "cross section the reference caches per (cell, group) and cycle not counted); log / sin / "
                     "cos / exp calls counted apart; counted by oracle/qs_oracle.c")
    data["generated_by"] = "python tests/golden/count_fp64_work.py"
    data.setdefault("workloads", {})
    for name in names:
        data["workloads"][name] = count_workload(name)
        print(name, data["workloads"][name])
    OUT.write_text(json.dumps(data, indent=2) + "\n")


if __name__ == "__main__":
    main(sys.argv[1:])
