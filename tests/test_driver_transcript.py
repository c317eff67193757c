"""The command-line driver's whole printout for a CORAL2-style deck against
the reference's own (tests/golden/transcript_out.npz, make_golden.py
--transcript: t_coral1 run with ``-e spectrum``), with the oracle standing
in for the GPU under the driver's loop (tests/helpers.OracleMonteCarlo):
after the deck echo, the same lines in the same order -- initMC's progress
lines text for text, per
cycle the counters and scalar-flux total as the reference prints them, the
cumulative timer table line for line (times and the reference's per-vault
call counts aside), the figure-of-merit line, and the four CORAL2 checks
text for text, fluence verdict and percentage included -- and the energy
spectrum file byte for byte; and ``-h`` printing the reference's argument
list text for text and stopping with its exit status."""
import numpy as np

from helpers import DECKS, OracleMonteCarlo

GOLD = np.load(DECKS.parent.parent / "tests" / "golden" / "transcript_out.npz")
TIMED_ALIKE = ("main", "cycleInit", "cycleTracking", "cycleFinalize", "cycleTracking_Test_Done")


def test_driver_transcript_matches_reference(monkeypatch, capsys, tmp_path):
    import quicksilver_gb300.__main__ as M
    monkeypatch.setattr(M, "MonteCarlo", OracleMonteCarlo)
    monkeypatch.setattr(M, "mc_sync", lambda tracker: None)
    stem = tmp_path / "spectrum"
    assert M.main([str(DECKS / "t_coral1.inp"), "-e", str(stem)]) == 0
    out = capsys.readouterr().out
    got = out[out.index("Building partition 0"):].split("\n")
    want = str(GOLD["stdout"]).split("\n")
    assert len(got) == len(want)
    timers = False
    for g, w in zip(got, want):
        gf, wf = g.split(), w.split()
        assert gf[:1] == wf[:1] and len(g) == len(w), (g, w)
        if g.startswith("Timer"):
            timers = True
        elif g.startswith("Figure Of Merit"):
            timers = False
        elif not timers and g[:8].strip().isdigit():       # summary line: counters and flux
            assert gf[:14] == wf[:14], (g, w)
        elif timers and gf and gf[0] in TIMED_ALIKE:
            assert gf[1] == wf[1], (g, w)
        elif not timers and not g.startswith(("cycle ", "Figure Of Merit")):
            assert g == w                                   # the CORAL2 check text
    assert (tmp_path / "spectrum.dat").read_text() == str(GOLD["spectrum"])


def test_help_lists_the_reference_arguments(capsys):
    import quicksilver_gb300.__main__ as M
    assert M.main(["-h"]) == 2
    out = capsys.readouterr().out
    assert out.startswith(str(GOLD["help"])) and "--exponential-tally" in out[len(str(GOLD["help"])):]
