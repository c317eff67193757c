"""The crossSectionsOut file (observe.cross_section_table, written by the
driver when the deck names one) against the file the unmodified reference's
initMC writes for the same decks (initMC.cc:392-490;
tests/golden/xsec_out.npz, make_golden.py --xsec): text for text."""
import numpy as np
import pytest

from helpers import DECKS
from quicksilver_gb300 import Deck
from quicksilver_gb300.observe import cross_section_table, write_cross_sections

XSEC = np.load(DECKS.parent.parent / "tests" / "golden" / "xsec_out.npz")


@pytest.mark.parametrize("name", sorted(XSEC.keys()))
def test_cross_section_file_matches_reference(name):
    deck = Deck.from_file(DECKS / f"{name}.inp")
    assert cross_section_table(deck.build(), deck.material_names) == str(XSEC[name])


def test_driver_keys_and_file(tmp_path):
    deck = Deck.from_file(DECKS / "t_nonflat.inp", {"crossSectionsOut": str(tmp_path / "xs")})
    assert deck.cross_sections_out == str(tmp_path / "xs")
    assert deck.material_names == sorted(deck.material_names)
    path = write_cross_sections(deck.cross_sections_out, deck.build(), deck.material_names)
    assert open(path).read() == str(XSEC["t_nonflat"])
