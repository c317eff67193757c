"""The oracle in the mode of the reference built with -DEXPONENTIAL_TALLY
(CycleTracking.cc:48-50: before every segment one random number r is drawn
from the particle's stream and exp(r) added to its cell's tally, which
cycleFinalize resets) against golden vectors from that build of the
unmodified reference (tests/golden/make_golden.py --exponential-tally).
The extra draw shifts every later random number, so the counters and census
particles pin the draw's place in the stream; the cell tally itself agrees
to summation order (both sides use the host's exp)."""
import hashlib

import numpy as np
import pytest

from helpers import DECKS, assert_flux_close, load_problem, oracle_run, sort_particles

GOLDEN = DECKS.parent.parent / "tests" / "golden"


def _sha(recs):
    return hashlib.sha256(np.ascontiguousarray(recs).tobytes()).hexdigest()


@pytest.mark.parametrize("name", ["t_homog", "t_fission"])
def test_oracle_exponential_tally_matches_reference(name):
    gold = np.load(GOLDEN / f"exp_{name}.npz")
    _, sim, hp = load_problem(f"{name}.inp")
    run = oracle_run(hp, sim)
    run.enable_exponential_tally()
    plain = np.load(GOLDEN / f"{name}.npz")["balance"]
    for c in range(gold["balance"].shape[0]):
        run.cycle_init()
        run.cycle_tracking(4)
        bal = run.balance()
        bal[4] = len(run.processed())
        np.testing.assert_array_equal(bal, gold["balance"][c], err_msg=f"cycle {c} balance")
        assert_flux_close(run.flux().sum(axis=1), gold["flux_cell"][c])
        assert_flux_close(run.cell_tally(), gold["cell_tally"][c])
        cen = sort_particles(run.processed())
        assert len(cen) == gold["census_n"][c] and _sha(cen) == gold["census_sha"][c]
        run.cycle_finalize()
        assert not run.cell_tally().any()   # reset every cycle, as Tallies.cc:91 does
    # the extra draw changes the histories: the counters differ from the default build's
    assert not np.array_equal(gold["balance"], plain[: len(gold["balance"])])
    # mean of exp(U) over (0, 1) is e - 1
    per_segment = gold["cell_tally"].sum() / gold["balance"][:, 12].sum()
    assert abs(per_segment - (np.e - 1)) < 0.01


def test_one_shot_tracking_with_cell_tally():
    import oracle_py as O
    _, sim, hp = load_problem("t_homog.inp")
    run = oracle_run(hp, sim)
    run.cycle_init()
    parts = run.processing()
    census, bal, flux, ct = O.track(hp.ptr, hp.num_cells, hp.num_groups, parts, cell_tally=True)
    run.enable_exponential_tally()
    run.cycle_tracking(4)
    np.testing.assert_array_equal(bal[[0, 1, 2, 3, 5, 6, 7, 12]], run.balance()[[0, 1, 2, 3, 5, 6, 7, 12]])
    assert_flux_close(ct, run.cell_tally())
    assert_flux_close(flux, run.flux())
