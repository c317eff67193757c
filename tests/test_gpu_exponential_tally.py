"""The reference's -DEXPONENTIAL_TALLY build on the GPU
(qsg_set_exponential_tally): before every segment one random number r is
drawn from the particle's stream and exp(r) added to its cell's tally.

* One tracking call against the oracle in that mode on the same particles:
  counters bit for bit, cell tally and flux per cell within 1e-12 (CUDA's exp
  and the host's may differ in the last bit; the draw itself is exact).
* Whole device cycles against the oracle and against the golden counters of
  the reference built with the define: counters bit for bit every cycle, the
  cycle's cell tally within 1e-12, reset by cycle finalize.
* Switching it off restores the default build's counters; the captured-cycle
  path carries it; reading it while off is an error.
"""
import numpy as np
import pytest

import oracle_py as O
from helpers import DECKS, assert_flux_close, load_problem, oracle_run
from quicksilver_gb300 import _native as N
from quicksilver_gb300.monte_carlo import MonteCarlo
from quicksilver_gb300.tracker import Tracker

pytestmark = pytest.mark.gpu

GOLDEN = DECKS.parent.parent / "tests" / "golden"
SLOTS = [0, 1, 2, 3, 5, 6, 7, 12]   # the counters tracking itself sets


@pytest.mark.parametrize("name", ["t_homog.inp", "t_fission.inp", "t_nonflat.inp"])
def test_tracking_with_exponential_tally_matches_oracle(gpu, name):
    _, sim, hp = load_problem(name)
    run = oracle_run(hp, sim)
    run.cycle_init()
    parts = run.processing()
    _, want_bal, want_flux, want_ct = O.track(hp.ptr, hp.num_cells, hp.num_groups, parts, cell_tally=True)
    trk = Tracker(hp)
    try:
        trk.set_exponential_tally(True)
        trk.set_particles(parts)
        trk.track()
        bal, flux = trk.tallies()
        np.testing.assert_array_equal(bal[SLOTS], want_bal[SLOTS])
        assert_flux_close(trk.cell_tally(), want_ct, rel=1e-12, scale_floor=1e-12)
        assert_flux_close(flux.sum(axis=1), want_flux.sum(axis=1), rel=1e-12, scale_floor=1e-12)
        assert abs(trk.cell_tally().sum() / bal[12] - (np.e - 1)) < 0.02
        trk.reset_tallies()
        assert not trk.cell_tally().any()
        assert trk.device_status() == 0
    finally:
        trk.close()


@pytest.mark.parametrize("name", ["t_homog", "t_fission"])
@pytest.mark.parametrize("use_graph", [False, True])
def test_device_cycles_with_exponential_tally(gpu, name, use_graph):
    deck, sim, hp = load_problem(f"{name}.inp")
    gold = np.load(GOLDEN / f"exp_{name}.npz")
    cycles = gold["balance"].shape[0]
    run = oracle_run(hp, sim)
    run.enable_exponential_tally()
    # captured cycles run a fixed number of tracking passes over stores that
    # cannot grow between them: enough of both for the fission deck, whose
    # census grows to ~3e5
    mc = MonteCarlo(deck, problem=hp, max_passes=64, store_capacity=4 * int(gold["census_n"].max()) + 4096)
    try:
        mc.exponential_tally(True)
        if use_graph:
            mc.run_cycles(cycles, use_graph=True)
            hist = mc.history(0, cycles)
            np.testing.assert_array_equal(hist.balance, gold["balance"])
            assert not mc.cell_tally().any()   # reset by the last cycle finalize
        else:
            for c in range(cycles):
                run.cycle_init()
                mc.cycle_init()
                run.cycle_tracking(0)
                mc.cycle_tracking()
                assert_flux_close(mc.cell_tally(), run.cell_tally(), rel=1e-12, scale_floor=1e-12)
                assert_flux_close(mc.cell_tally(), gold["cell_tally"][c], rel=1e-12, scale_floor=1e-12)
                run.cycle_finalize()
                mc.cycle_finalize()
                assert not mc.cell_tally().any()
                hist = mc.history(c, 1)
                np.testing.assert_array_equal(hist.balance[0], run.last_balance(), err_msg=f"cycle {c} vs oracle")
                np.testing.assert_array_equal(hist.balance[0], gold["balance"][c], err_msg=f"cycle {c} vs reference")
        assert mc.device_status() == 0
    finally:
        mc.close()


def test_exponential_tally_off_restores_default_build(gpu):
    deck, sim, hp = load_problem("t_homog.inp")
    mc = MonteCarlo(deck, problem=hp)
    try:
        mc.exponential_tally(True)
        mc.exponential_tally(False)
        with pytest.raises(N.QsgError):
            mc.cell_tally()
        h = mc.run(3)
        np.testing.assert_array_equal(h.balance, np.load(GOLDEN / "t_homog.npz")["balance"][:3])
        assert N.lib().qsg_set_exponential_tally(mc.tracker.handle, 2) == N.QSG_ERR_INVALID
    finally:
        mc.close()
