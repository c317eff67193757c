"""GB300-native cycle tracking for Quicksilver decks.

Public API (mirrors the reference's MonteCarlo / cycle driver, main.cc:38-324):

    from quicksilver_gb300 import Deck, MonteCarlo
    mc = MonteCarlo(Deck.from_file("problem.inp"))
    for _ in range(mc.n_steps):
        mc.cycle_init(); mc.cycle_tracking(); mc.cycle_finalize()

The tracking runs in hand-written sm_103a CUDA (libqsg.so); there is no CPU
fallback.
"""
from .problem import Deck, HostProblem  # noqa: F401
from ._native import BALANCE_FIELDS, PARTICLE_DTYPE, QsgError  # noqa: F401

__all__ = ["Deck", "HostProblem", "BALANCE_FIELDS", "PARTICLE_DTYPE", "QsgError"]
