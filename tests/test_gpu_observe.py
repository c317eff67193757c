"""GPU observability tallies (qsg_set_observers) and the command-line driver
against the oracle's run with the reference's observers restated
(tests/test_observe.py): fluence per cell to summation order, census energy
spectrum and cumulative counters exactly, the same CORAL2 verdicts."""
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

from helpers import DECKS, assert_flux_close
from quicksilver_gb300 import Deck
from quicksilver_gb300 import _native as N
from quicksilver_gb300.monte_carlo import BatchMonteCarlo, MonteCarlo
from quicksilver_gb300.observe import coral_benchmark_correctness, cumulative_balance
from test_observe import oracle_observe

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parent.parent


@pytest.mark.parametrize("name", ["t_coral1.inp", "t_fission.inp", "t_homog.inp"])
def test_gpu_observers_match_oracle(gpu, name):
    hist, fluence, spectrum, _ = oracle_observe(name)
    mc = MonteCarlo(Deck.from_file(DECKS / name))
    try:
        mc.observe(fluence=True, spectrum=True)
        h = mc.run()
        np.testing.assert_array_equal(h.balance[:, [0, 1, 2, 3, 5, 6, 7, 12]], hist[:, [0, 1, 2, 3, 5, 6, 7, 12]])
        assert_flux_close(mc.fluence(), fluence, rel=1e-12, scale_floor=1e-12)
        np.testing.assert_array_equal(mc.energy_spectrum()[0], spectrum)
        a = coral_benchmark_correctness(cumulative_balance(h.balance), mc.fluence(), 1, out=None)
        b = coral_benchmark_correctness(cumulative_balance(hist), fluence, 1, out=None)
        assert a == b
    finally:
        mc.close()


def test_gpu_spectrum_per_problem_in_a_batch(gpu):
    deck = Deck.from_file(DECKS / "t_coral1.inp")
    single = MonteCarlo(deck)
    single.observe(spectrum=True)
    single.run()
    want = single.energy_spectrum()[0]
    single.close()
    # the deck's fission chains need more tracking passes per cycle than the
    # default of 8 that a captured cycle runs
    bmc = BatchMonteCarlo([deck, deck], seed_offsets=[0, 777], max_passes=64)
    try:
        bmc.observe(spectrum=True)
        h = bmc.run(deck.simulation.n_steps, use_graph=True)
        spec = bmc.energy_spectrum()
        np.testing.assert_array_equal(spec[0], want)
        assert spec[1].sum() == h.balance[:, 1, N.BAL["census"]].sum()
    finally:
        bmc.close()


def test_gpu_command_line_driver(gpu, tmp_path):
    stem = tmp_path / "spectrum"
    res = subprocess.run([sys.executable, "-m", "quicksilver_gb300", str(DECKS / "t_coral1.inp"),
                          "--energySpectrum", str(stem)], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert res.returncode == 0, res.stderr
    out = res.stdout
    assert "Figure Of Merit" in out and "[Num Segments / Cycle Tracking Time]" in out
    assert "PASS:: No Particles Lost During Run" in out
    assert "PASS:: Absorption / Fission / Scatter Ratios maintained" in out
    rows = [l.split() for l in out.splitlines() if l.strip() and l.split()[0].isdigit()]
    assert len(rows) == Deck.from_file(DECKS / "t_coral1.inp").simulation.n_steps
    counts = [int(l.split("\t")[2]) for l in open(str(stem) + ".dat").read().splitlines()]
    census = sum(int(r[11]) for r in rows)
    assert sum(counts) == census


def test_gpu_command_line_driver_exponential_tally(gpu):
    """--exponential-tally: the per-cycle counters the driver prints are those
    of the reference built with -DEXPONENTIAL_TALLY, and so are the cell-tally
    totals (to summation order and CUDA's exp)."""
    res = subprocess.run([sys.executable, "-m", "quicksilver_gb300", str(DECKS / "t_homog.inp"),
                          "--exponential-tally"], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert res.returncode == 0, res.stderr
    gold = np.load(ROOT / "tests" / "golden" / "exp_t_homog.npz")
    rows = [l.split() for l in res.stdout.splitlines() if l.strip() and l.split()[0].isdigit()]
    assert len(rows) == len(gold["balance"])
    cols = ["start", "source", "rr", "split", "absorb", "scatter", "fission", "produce", "collision", "escape",
            "census", "num_segments"]
    for c, r in enumerate(rows):
        for k, name in enumerate(cols):
            assert int(r[1 + k]) == int(gold["balance"][c][N.BAL[name]]), (c, name)
        want = gold["cell_tally"][c].sum()
        assert abs(float(r[-1]) - want) <= 1e-6 * want   # printed with 7 significant digits


def test_gpu_command_line_driver_cycle_timers(gpu):
    """-c 1 (cycleTimers): after every summary line the driver prints the
    reference's last-cycle timer table, then the cumulative one; the lines
    line up with the reference's own printout of the same run
    (tests/golden/timers_out.npz), and so do the call counts of the timers
    both sides time alike (main, cycleInit, cycleTracking, cycleFinalize and
    the done test)."""
    res = subprocess.run([sys.executable, "-m", "quicksilver_gb300", str(DECKS / "t_homog.inp"), "-c", "1"],
                         cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert res.returncode == 0, res.stderr
    got = res.stdout[res.stdout.index("cycle "):].split("\n")
    want = str(np.load(ROOT / "tests" / "golden" / "timers_out.npz")["t_homog"]).split("\n")
    assert len(got) == len(want)
    for g, w in zip(got, want):
        assert len(g) == len(w) and g.split()[:1] == w.split()[:1], (g, w)
        if g.split()[:1] and g.split()[0] in ("main", "cycleInit", "cycleTracking", "cycleFinalize",
                                              "cycleTracking_Test_Done"):
            assert g.split()[1] == w.split()[1], (g, w)
