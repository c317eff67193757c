"""The driver's timer reports (quicksilver_gb300.__main__.timer_table /
timer_report) against the reference's own printout of t_homog run with
``-c 1`` (tests/golden/timers_out.npz, make_golden.py --timers): every
last-cycle table (MC_Fast_Timer.cc:106-152) and the cumulative table with the
figure of merit (MC_Fast_Timer.cc:58-104), text for text, when given the
reference's own call counts and microseconds; and the driver's whole loop on
the CPU (the oracle standing in for the GPU) printing the reference's lines
in the reference's order."""
import io

import numpy as np

from helpers import DECKS, OracleMonteCarlo
from quicksilver_gb300.__main__ import TIMERS, timer_report, timer_table

TEXT = str(np.load(DECKS.parent.parent / "tests" / "golden" / "timers_out.npz")["t_homog"])


def blocks(kind: str):
    """Each table of that kind as (its text from the blank line on, {name: (calls, seconds)})."""
    lines = TEXT.split("\n")
    out = []
    for i, line in enumerate(lines):
        if line.startswith("Timer") and kind in line:
            body = lines[i + 3:i + 3 + len(TIMERS)]
            clock = {}
            for row in body:
                f = row.split()
                # whole microseconds, given back as seconds half a microsecond
                # above so that flooring returns them
                clock[f[0]] = (int(f[1]), (float(f[3]) + 0.5) * 1e-6)
            out.append(("\n".join([""] + lines[i:i + 3 + len(TIMERS)]) + "\n", clock))
    return out


def test_last_cycle_tables_match_reference():
    tables = blocks("Last Cycle")
    assert len(tables) == 3
    for cycle, (want, clock) in enumerate(tables):
        assert list(clock) == TIMERS
        buf = io.StringIO()
        timer_table(buf, "Last Cycle", clock)
        assert buf.getvalue() == want
        # what the reference counts: main not yet stopped, cycleFinalize
        # stopped and restarted around the summary line, no done test
        assert clock["main"][0] == 0 and clock["cycleTracking_Test_Done"][0] == 0
        assert clock["cycleInit"][0] == clock["cycleTracking"][0] == cycle + 1
        assert clock["cycleFinalize"][0] == 2 * (cycle + 1)


def test_cumulative_table_and_figure_of_merit_match_reference():
    (want, clock), = blocks("Cumulative")
    summary = [l.split() for l in TEXT.split("\n") if l[:8].strip().isdigit()]
    num_segments = sum(int(r[12]) for r in summary)
    buf = io.StringIO()
    timer_report(buf, {k: list(v) for k, v in clock.items()}, num_segments)
    fom = next(l for l in TEXT.split("\n") if l.startswith("Figure Of Merit"))
    assert buf.getvalue() == want + fom + "\n"


def test_driver_prints_reference_layout(monkeypatch, capsys):
    """The driver run with -c 1 prints, from its summary header on, the lines
    the reference prints for the same run: the same line count, each line as
    long as the reference's with the same first field, and the same call
    counts for the timers both sides time alike."""
    import quicksilver_gb300.__main__ as M
    monkeypatch.setattr(M, "MonteCarlo", OracleMonteCarlo)
    monkeypatch.setattr(M, "mc_sync", lambda tracker: None)
    assert M.main([str(DECKS / "t_homog.inp"), "-c", "1"]) == 0
    out = capsys.readouterr().out
    got = out[out.index("cycle "):].split("\n")
    want = TEXT.split("\n")
    assert len(got) == len(want)
    for g, w in zip(got, want):
        assert len(g) == len(w) and g.split()[:1] == w.split()[:1], (g, w)
        if g.split()[:1] and g.split()[0] in ("main", "cycleInit", "cycleTracking", "cycleFinalize",
                                              "cycleTracking_Test_Done"):
            assert g.split()[1] == w.split()[1], (g, w)
        if g[:8].strip().isdigit():   # summary lines: the counters and flux as the reference prints them
            assert g.split()[:14] == w.split()[:14]
