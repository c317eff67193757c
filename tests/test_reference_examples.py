"""Every example deck the reference ships reads through this library's deck
reader as the reference reads it: our start-up echo (qsg_deck_write) equals,
text for text, the echo the unmodified reference prints for the same file
(the harness built from its sources, QS_ECHO), and each deck builds a
problem that passes qsg_create's checks, the reference's mesh self-test
included.  Runs where the reference's sources and the harness built from
them are present (they are test infrastructure; nothing of the decks is
kept in this repository), and skips elsewhere."""
import ctypes
import os
import subprocess
from pathlib import Path

import pytest

from quicksilver_gb300 import Deck
from quicksilver_gb300 import _native as N

ROOT = Path(__file__).resolve().parent.parent
import __graft_entry__ as _entry   # noqa: E402  (its REF_SRC names the reference's sources)

EXAMPLES = _entry.REF_SRC.parent / "Examples"
HARNESS = ROOT / "oracle" / "_ref" / "qs_ref_harness"
DECKS = sorted(EXAMPLES.rglob("*.inp")) if EXAMPLES.exists() else []

pytestmark = pytest.mark.skipif(not DECKS or not HARNESS.exists(),
                                reason="the reference's sources or the harness built from them are absent")


def _reference_echo(deck: Path, tmp_path: Path) -> str:
    out = tmp_path / "echo.txt"
    env = dict(os.environ, QS_ECHO=str(out), QS_ECHO_ONLY="1")
    res = subprocess.run([str(HARNESS), "-i", str(deck)], env=env, capture_output=True, text=True, timeout=120)
    assert res.returncode == 0, res.stderr[-2000:]
    return out.read_text()


@pytest.mark.parametrize("deck", DECKS, ids=[str(d.relative_to(EXAMPLES)) for d in DECKS])
def test_reference_example_deck_reads_the_same(deck, tmp_path):
    ours = Deck.from_file(deck)
    assert ours.text() == _reference_echo(deck, tmp_path)


@pytest.mark.parametrize("deck", [d for d in DECKS if "4096" not in d.name and "_36" not in d.name],
                         ids=lambda d: d.name)
def test_reference_example_deck_builds_a_valid_problem(deck):
    hp = Deck.from_file(deck, {"nx": 4, "ny": 4, "nz": 4}).build()   # mesh kept small; the tables' kind is the deck's
    assert N.lib().qsg_problem_check(ctypes.byref(hp.view)) == N.QSG_OK, N.last_error()
