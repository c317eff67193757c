"""Error behaviour of the C ABI on a GPU host: invalid arguments come back as
QSG_ERR_* codes with a message (the reference's qs_assert only prints and
continues, qs_assert.hh:9-26), and the handle stays usable afterwards."""
import numpy as np
import pytest

from helpers import DECKS
from quicksilver_gb300 import Deck
from quicksilver_gb300 import _native as N
from quicksilver_gb300.monte_carlo import MonteCarlo
from quicksilver_gb300.sensitivity import ABSORPTION, Param, band_params

pytestmark = pytest.mark.gpu


def _mc():
    return MonteCarlo(Deck.from_file(DECKS / "t_sens.inp"))


def test_sensitivity_argument_errors(gpu):
    mc = _mc()
    try:
        trk = mc.tracker
        G = trk.num_groups
        cases = [
            [Param(0, ABSORPTION, 0, G), Param(0, ABSORPTION, 3, 5)],          # overlapping entries
            [Param(7, ABSORPTION, 0, G)],                                       # material out of range
            [Param(0, 5, 0, G)],                                                # reaction type out of range
            [Param(0, ABSORPTION, 3, 3)],                                       # empty group range
            [Param(0, ABSORPTION, 0, G, theta=0.0)],                            # theta must be positive
            [Param(0, ABSORPTION, 0, 1)] * 0 + [Param(m % 3, 1 + (m % 2), 0, G) for m in range(40)],  # > 32 params
        ]
        for params in cases:
            with pytest.raises(N.QsgError) as exc:
                trk.enable_sensitivity(params)
            assert exc.value.code == N.QSG_ERR_INVALID and str(exc.value)
        # the handle still works: a valid set, then a run
        trk.enable_sensitivity(band_params(mc.problem.array("energies"), mc.problem.num_materials))
        h = mc.run(1)
        assert h.segments() > 0 and trk.read_sensitivity()["flux_cell"].sum() > 0
    finally:
        mc.close()


def test_tuning_and_kernel_argument_errors(gpu):
    mc = _mc()
    try:
        lib, h = N.lib(), mc.tracker.handle
        calls = [(lib.qsg_set_tuning, (96, 0, 0), "block size"),
                 (lib.qsg_set_track_kernel, (2,), "kind"),
                 (lib.qsg_set_observers, (8,), "flag"),
                 (lib.qsg_set_pool_tuning, (33, 0), "collision step"),
                 (lib.qsg_set_pool_tuning, (0, 65), "refill")]
        for fn, args, words in calls:
            assert fn(h, *args) == N.QSG_ERR_INVALID
            assert words in N.last_error()
        with pytest.raises(N.QsgError):
            mc.fluence()            # observers are off
        assert mc.run(1).segments() > 0
    finally:
        mc.close()


def test_store_overflow_is_flagged(gpu):
    """Stores sized below the population (store_capacity far too small) in
    the captured-cycle path, which cannot grow them between passes: the
    writers drop what does not fit, readers stop at the capacity, and the run
    reports QSG_DEV_STORE_OVERFLOW instead of corrupting memory.  (The
    host-driven path grows the stores as needed.)"""
    deck = Deck.from_file(DECKS / "t_fission.inp")   # ~7e4 census particles per cycle
    mc = MonteCarlo(deck, store_capacity=64)
    try:
        mc.run_cycles(2, use_graph=True)
        mc.history(0, 2)                     # waits for the device
        assert mc.device_status() & N.QSG_DEV_STORE_OVERFLOW
    finally:
        mc.close()
