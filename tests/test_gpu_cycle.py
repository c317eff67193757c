"""Whole cycles on the device (qsg_cycle_init / qsg_track_cycle /
qsg_cycle_finalize) against the C oracle's cycleInit / cycleTracking /
cycleFinalize, and against the reference's golden counters.

All 13 balance counters must agree bit for bit every cycle (START, SOURCE,
RR and SPLIT pin the device-side source, population control and roulette).
The particle set produced by the device cycle init must match the oracle's:
integer fields (seeds, identifiers, cells) exactly, floating-point fields to
1e-12 relative (the isotropic direction and the sampled number of mean free
paths go through cos/sin/log).  The scalar-flux total per cycle within 1e-12.
"""
import numpy as np
import pytest

from helpers import DECKS, load_problem, oracle_run, sort_particles
from quicksilver_gb300.monte_carlo import MonteCarlo

pytestmark = pytest.mark.gpu

GOLDEN = DECKS.parent.parent / "tests" / "golden"
INT_FIELDS = ["random_number_seed", "identifier", "last_event", "num_collisions", "breed", "species", "domain", "cell"]
FP_FIELDS = ["x", "y", "z", "vx", "vy", "vz", "kinetic_energy", "weight", "time_to_census", "age",
             "num_mean_free_paths", "num_segments"]
DECK_NAMES = ["t_homog", "t_absorb", "t_escape", "t_nocoll", "t_scatter_octant", "t_fission", "t_nonflat",
              "t_default", "config1"]


def compare_sets(got, want, rtol):
    assert len(got) == len(want)
    g, w = sort_particles(got), sort_particles(want)
    for f in INT_FIELDS:
        np.testing.assert_array_equal(g[f], w[f], err_msg=f)
    for f in FP_FIELDS:
        np.testing.assert_allclose(g[f], w[f], rtol=rtol, atol=0, err_msg=f)


@pytest.mark.parametrize("name", DECK_NAMES)
def test_device_cycles_match_oracle_and_reference(gpu, name):
    deck, sim, hp = load_problem(f"{name}.inp")
    run = oracle_run(hp, sim)
    mc = MonteCarlo(deck, problem=hp)
    gold = np.load(GOLDEN / f"{name}.npz")["balance"]
    for c in range(sim.n_steps):
        run.cycle_init()
        mc.cycle_init()
        if c == 0:
            # same inputs: the first cycle's particles come from the source alone
            compare_sets(mc.processing(), run.processing(), rtol=1e-12)
        else:
            assert mc.tracker.sizes()[0] == run.processing().shape[0]
        mc.cycle_tracking()
        mc.cycle_finalize()
        run.cycle_tracking(0)
        want_flux_total = run.flux().sum()
        run.cycle_finalize()
        hist = mc.history(c, 1)
        np.testing.assert_array_equal(hist.balance[0], run.last_balance(), err_msg=f"{name} cycle {c} vs oracle")
        np.testing.assert_array_equal(hist.balance[0], gold[c], err_msg=f"{name} cycle {c} vs reference")
        assert abs(hist.flux_total[0] - want_flux_total) <= 1e-12 * abs(want_flux_total)
    assert mc.device_status() == 0
    mc.close()


def test_device_run_config1_matches_reference(gpu):
    deck, sim, hp = load_problem("config1.inp")
    mc = MonteCarlo(deck, problem=hp)
    hist = mc.run()
    gold = np.load(GOLDEN / "config1.npz")
    np.testing.assert_array_equal(hist.balance, gold["balance"])
    np.testing.assert_allclose(hist.flux_total, gold["flux_total"], rtol=1e-12)
    mc.close()
