"""The driver's per-cycle summary (quicksilver_gb300.__main__.summary_header
/ summary_line) against the reference's own Tallies::PrintSummary output for
the same decks (Tallies.cc:122-144; tests/golden/summary_out.npz,
make_golden.py --summary): the header text for text, and on every cycle the
cycle number, the 12 counters and the scalar-flux sum as printed (the
oracle's counters are bitwise the reference's); the three phase times
differ from run to run and are left out."""
import numpy as np
import pytest

from helpers import DECKS, load_problem, oracle_run
from quicksilver_gb300.__main__ import summary_header, summary_line

SUMMARY = np.load(DECKS.parent.parent / "tests" / "golden" / "summary_out.npz")


@pytest.mark.parametrize("name", sorted(SUMMARY.keys()))
def test_summary_lines_match_reference(name):
    ref = str(SUMMARY[name]).splitlines()
    assert summary_header() == ref[0]
    _, sim, hp = load_problem(f"{name}.inp")
    run = oracle_run(hp, sim)
    for c, line in enumerate(ref[1:]):
        run.cycle_init()
        run.cycle_tracking(8)
        flux_total = run.flux().sum()
        run.cycle_finalize()
        got = summary_line(c, run.last_balance(), flux_total, (0.0, 0.0, 0.0))
        assert got.split()[:14] == line.split()[:14], f"cycle {c}"
        assert len(got) == len(line)
