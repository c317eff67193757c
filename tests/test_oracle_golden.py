"""The C oracle against golden vectors produced by the unmodified reference.

Balance counters must match bit for bit every cycle; scalar flux per
(cell, group) within 1e-12 relative (the oracle's OpenMP threads change only
the summation order); the particle sets after cycleInit and after
cycleTracking must be bitwise identical to the reference's (sorted by
identifier), which pins the source, population control, roulette and the
whole tracking restatement.
"""
import hashlib

import numpy as np
import pytest

from helpers import DECKS, assert_flux_close, load_problem, oracle_run, sort_particles

GOLDEN = DECKS.parent.parent / "tests" / "golden"
SMALL_DECKS = sorted(p.stem for p in GOLDEN.glob("t_*.npz"))


def _sha(recs):
    return hashlib.sha256(np.ascontiguousarray(recs).tobytes()).hexdigest()


def _proj(cells, groups):
    return np.random.default_rng(20240601).uniform(0.5, 1.5, size=(4, cells * groups))


def run_against_golden(name, threads=4, deck=None):
    gold = np.load(GOLDEN / f"{name}.npz")
    if deck is None:
        _, sim, hp = load_problem(f"{name}.inp")
    else:
        sim, hp = deck.simulation, deck.build()
    run = oracle_run(hp, sim)
    cycles = gold["balance"].shape[0]
    w = _proj(hp.num_cells, hp.num_groups)
    for c in range(cycles):
        run.cycle_init()
        ini = sort_particles(run.processing())
        assert len(ini) == gold["init_n"][c]
        assert _sha(ini) == gold["init_sha"][c], f"cycle {c}: particles after cycleInit differ"
        if c == 0:
            assert np.array_equal(ini[:32], gold["init_head"])
        run.cycle_tracking(threads)
        bal = run.balance()
        bal[4] = len(run.processed())
        np.testing.assert_array_equal(bal, gold["balance"][c], err_msg=f"cycle {c} balance")
        flux = run.flux()
        if "flux" in gold:
            assert_flux_close(flux, gold["flux"][c])
        if "flux_cell" in gold:
            assert_flux_close(flux.sum(axis=1), gold["flux_cell"][c])
        assert_flux_close(flux.sum(axis=0), gold["flux_group"][c])
        assert_flux_close(w @ flux.ravel(), gold["flux_proj"][c])
        cen = sort_particles(run.processed())
        assert _sha(cen) == gold["census_sha"][c], f"cycle {c}: census particles differ"
        run.cycle_finalize()
    assert run.warnings() == 0


@pytest.mark.parametrize("name", SMALL_DECKS)
def test_oracle_matches_reference_small(name):
    run_against_golden(name)


def test_oracle_matches_reference_config1():
    run_against_golden("config1", threads=8)


def test_oracle_matches_reference_config2():
    """The benchmark deck's first three cycles (43.8 M segments)."""
    run_against_golden("config2", threads=8)


def test_oracle_matches_reference_config4():
    """The differentiated workload's deck (escape boundaries), first three cycles."""
    run_against_golden("config4", threads=8)


def test_limit_invariants():
    """Analytic invariants of the limit decks (cf. the reference's example physics)."""
    B = {n: i for i, n in enumerate(("absorb", "census", "escape", "collision", "end", "fission", "produce",
                                     "scatter", "start", "source", "rr", "split", "num_segments"))}
    g = np.load(GOLDEN / "t_absorb.npz")["balance"]
    assert (g[:, B["absorb"]] == g[:, B["source"]] + g[:, B["split"]] + g[:, B["start"]] - g[:, B["rr"]]).all()
    assert (g[:, B["collision"]] == g[:, B["num_segments"]]).all()
    g = np.load(GOLDEN / "t_escape.npz")["balance"]
    assert (g[:, B["collision"]] == 0).all()
    g = np.load(GOLDEN / "t_nocoll.npz")["balance"]
    assert (g[:, B["collision"]] == 0).all() and (g[:, B["escape"]] == 0).all()
    g = np.load(GOLDEN / "t_scatter_octant.npz")["balance"]
    assert (g[:, B["absorb"]] == 0).all() and (g[:, B["collision"]] == g[:, B["scatter"]]).all()
    g = np.load(GOLDEN / "t_fission.npz")["balance"]
    assert (g[:, B["fission"]] > 0).all() and (g[:, B["produce"]] > 0).all()
    # particle conservation (CoralBenchmark.cc:152-174)
    for name in SMALL_DECKS + ["config1"]:
        g = np.load(GOLDEN / f"{name}.npz")["balance"].astype(np.int64)
        gains = g[:, B["start"]] + g[:, B["source"]] + g[:, B["produce"]] + g[:, B["split"]]
        losses = g[:, B["absorb"]] + g[:, B["census"]] + g[:, B["escape"]] + g[:, B["rr"]] + g[:, B["fission"]]
        np.testing.assert_array_equal(gains, losses, err_msg=name)


def test_oracle_matches_reference_config5_replica():
    """config5's first replica (64^3 cells in five slabs, five materials,
    escape boundaries) at 3e6 particles, two cycles."""
    import re
    from quicksilver_gb300 import Deck
    from quicksilver_gb300.decks.make_decks import config5
    deck = Deck.from_string(re.sub(r"nSteps: \d+", "nSteps: 2", config5(n_particles=3_000_000)[0]))
    run_against_golden("config5_r0", threads=8, deck=deck)


@pytest.mark.parametrize("problem", [4, 6, 15, 26, 33])
def test_oracle_matches_reference_config3_problem(problem):
    """Problems of the config3 ensemble, one per mesh edge (48 / 32 / 24 / 8 /
    16; problem 4 sources nothing: fewer particles than the per-cell floor
    needs), two cycles with the reference's own seeding."""
    import re
    from quicksilver_gb300 import Deck
    from quicksilver_gb300.decks.make_decks import config3
    deck = Deck.from_string(re.sub(r"nSteps: \d+", "nSteps: 2", config3()[problem]))
    run_against_golden(f"config3_p{problem:02d}", threads=8, deck=deck)
