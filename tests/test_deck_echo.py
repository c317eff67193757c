"""The deck echo (qsg_deck_write, Deck.text) against the reference's own
start-up echo of the same decks (printParameters, Parameters.cc:97-215;
tests/golden/deck_echo.npz from the unmodified reference, make_golden.py
--echo): text for text, every default filled in the same way.  The echo is
a replayable deck: parsed again it echoes the same and builds the same
tables."""
from pathlib import Path

import numpy as np
import pytest

from helpers import DECKS
from quicksilver_gb300 import Deck

GOLDEN = DECKS.parent.parent / "tests" / "golden"
ECHO = np.load(GOLDEN / "deck_echo.npz")


def _normalise(text: str) -> str:
    """The inputFile line records the path the deck was given; keep its file name."""
    out = []
    for line in text.splitlines():
        if line.startswith("   inputFile: "):
            line = "   inputFile: " + Path(line.split(": ", 1)[1]).name
        out.append(line)
    return "\n".join(out)


DECK_NAMES = sorted(k for k in ECHO.keys() if not k.startswith("cli_"))
COMMAND_LINES = sorted(k for k in ECHO.keys() if k.startswith("cli_") and not k.endswith("_args"))


@pytest.mark.parametrize("name", DECK_NAMES)
def test_echo_matches_reference(name):
    got = Deck.from_file(DECKS / f"{name}.inp").text()
    assert _normalise(got) == _normalise(str(ECHO[name]))


@pytest.mark.parametrize("name", COMMAND_LINES)
def test_command_line_matches_reference(name, monkeypatch):
    """The driver's flags, their precedence over / under the deck's keys and
    the default problem without a deck, as getParameters gives them: the
    echo of the same command line, text for text."""
    from quicksilver_gb300.__main__ import deck_from_command_line
    monkeypatch.chdir(DECKS.parent.parent)   # the command lines name decks relative to the repository
    deck, _ = deck_from_command_line([str(a) for a in ECHO[name + "_args"]])
    assert _normalise(deck.text()) == _normalise(str(ECHO[name]))


@pytest.mark.parametrize("name", ["t_homog", "t_fission", "t_nonflat", "config2"])
def test_echo_is_a_replayable_deck(name):
    deck = Deck.from_file(DECKS / f"{name}.inp")
    again = Deck.from_string(deck.text())
    # inputFile is the command line's (-i), in the reference too: a deck read
    # back from text has none
    drop = lambda t: "\n".join(l for l in t.splitlines() if not l.startswith("   inputFile:"))
    assert drop(again.text()) == drop(deck.text())
    if "shape: sphere" not in deck.text():   # the echo, like the reference's, leaves out a sphere's radius
        a, b = deck.build(), again.build()
        for table in ("cell_material", "cell_number_density", "facet_planes", "reaction_xs"):
            np.testing.assert_array_equal(a.array(table), b.array(table))
