"""CPU checks of batch construction (no GPU needed): the union builder's
validation errors surface through the C ABI before any device work."""
import ctypes

from helpers import DECKS
from quicksilver_gb300 import Deck
from quicksilver_gb300 import _native as N


def test_batch_rejects_mismatched_energy_grids(has_gpu):
    a = Deck.from_file(DECKS / "t_homog.inp").build()       # 16 groups
    b = Deck.from_file(DECKS / "t_nonflat.inp").build()     # 40 groups
    views = (N.QsgProblem * 2)(a.view, b.view)
    h = ctypes.c_void_p()
    rc = N.lib().qsg_batch_create(views, 2, None, ctypes.byref(h))
    assert rc == N.QSG_ERR_INVALID and "energy grid" in N.last_error()


def test_config3_decks_are_well_formed():
    from quicksilver_gb300.decks.make_decks import config3
    texts = config3()
    assert len(texts) == 64
    for t in texts[:6]:
        d = Deck.from_string(t)
        s = d.simulation
        assert s.nx in (8, 16, 24, 32, 48) and 1e4 <= s.n_particles <= 2e6 and s.n_groups == 230


def test_batch_union_passes_the_problem_checks(has_gpu):
    """The union of two problems (cells shifted into one numbering) passes
    qsg_create's checks, the facet-adjacency self-test included: without a
    GPU the call gets as far as looking for a device."""
    a = Deck.from_file(DECKS / "t_homog.inp").build()
    b = Deck.from_file(DECKS / "t_homog.inp", {"nx": 4, "ny": 4, "nz": 4, "lx": 4, "ly": 4, "lz": 4}).build()
    views = (N.QsgProblem * 2)(a.view, b.view)
    h = ctypes.c_void_p()
    rc = N.lib().qsg_batch_create(views, 2, None, ctypes.byref(h))
    if has_gpu:
        assert rc == N.QSG_OK, N.last_error()
        N.lib().qsg_destroy(h)
    else:
        assert rc == N.QSG_ERR_NO_DEVICE, N.last_error()
