"""The balance-counter identities that the full-size GPU runs are checked by
(tests/test_gpu_configs.py), shown to hold on the unmodified reference's own
counters: every golden deck, every cycle."""
import numpy as np
import pytest

from helpers import DECKS, balance_identities

GOLDEN = DECKS.parent.parent / "tests" / "golden"


@pytest.mark.parametrize("name", sorted(p.stem for p in GOLDEN.glob("t_*.npz")) + ["config1", "config2", "config4", "config5_r0"]
                         + sorted(p.stem for p in GOLDEN.glob("config3_p*.npz")))
def test_identities_hold_on_the_reference_counters(name):
    balance_identities(np.load(GOLDEN / f"{name}.npz")["balance"], name)


def test_identities_catch_a_broken_count():
    bal = np.load(GOLDEN / "t_fission.npz")["balance"].copy()
    bal[1, 0] += 1   # one absorption too many
    with pytest.raises(AssertionError):
        balance_identities(bal)
