"""The CORAL2 correctness checks (observe.coral_benchmark_correctness)
print, text for text, what the unmodified reference's
coralBenchmarkCorrectness prints (CoralBenchmark.cc:17-228;
tests/golden/coral_out.npz, make_golden.py --coral) for the same runs:
t_coral1 as written and t_homog / t_fission with coralBenchmark 1 / 2, so
that failing checks (with their infinite ratios) are pinned too.  Inputs:
the oracle's counters (bitwise the reference's) and fluence accumulated as
Fluence::compute does (Tallies.cc:100-118: per cycle, each cell's groups
in order)."""
import io

import numpy as np
import pytest

from helpers import DECKS, load_problem, oracle_run
from quicksilver_gb300.observe import coral_benchmark_correctness, cumulative_balance

CORAL = np.load(DECKS.parent.parent / "tests" / "golden" / "coral_out.npz")
RUNS = {"t_coral1": None, "t_homog": 1, "t_fission": 2}   # coralBenchmark set for the run (None: the deck's)


@pytest.mark.parametrize("name", sorted(CORAL.keys()))
def test_coral_checks_print_the_references_text(name):
    level = RUNS[name]
    deck, sim, hp = load_problem(f"{name}.inp", {"coralBenchmark": str(level)} if level else None)
    run = oracle_run(hp, sim)
    fluence = np.zeros(hp.num_cells)
    balances = []
    for _ in range(sim.n_steps):
        run.cycle_init()
        run.cycle_tracking(4)
        flux = run.flux()
        for g in range(flux.shape[1]):
            fluence += flux[:, g]
        run.cycle_finalize()
        balances.append(run.last_balance())
    out = io.StringIO()
    coral_benchmark_correctness(cumulative_balance(np.array(balances)), fluence, sim.coral_benchmark, out)
    assert out.getvalue() == str(CORAL[name])
