"""Shared helpers for the parity tests (test infrastructure)."""
from __future__ import annotations

import numpy as np

from quicksilver_gb300 import Deck
from quicksilver_gb300 import _native as N

DECKS = __import__("pathlib").Path(__file__).resolve().parent.parent / "quicksilver_gb300" / "decks"


def load_problem(deck_name: str, overrides: dict | None = None):
    deck = Deck.from_file(DECKS / deck_name, overrides)
    return deck, deck.simulation, deck.build()


def oracle_run(hp, sim):
    import oracle_py as O
    return O.OracleRun(hp.ptr, hp.num_cells, hp.num_groups, hp.source_rates(), sim.n_particles,
                       sim.e_min, sim.e_max, sim.low_weight_cutoff, sim.load_balance, keepalive=hp)


def sort_particles(recs: np.ndarray) -> np.ndarray:
    return recs[np.lexsort((recs["random_number_seed"], recs["identifier"]))]


def assert_flux_close(got: np.ndarray, want: np.ndarray, rel: float = 1e-12, scale_floor: float = 0.0):
    """Per (cell, group) agreement: |got - want| <= rel*|want| + scale_floor*mean(|want| over nonzero).

    With scale_floor = 0 this is a pure per-entry relative bound (used between
    two CPU runs with the same libm, where only summation order differs).  The
    GPU tests pass scale_floor = 1e-12: libdevice's log/sincos round
    differently from glibc in the last bit, which moves a trajectory by ~1e-15
    cm; on an entry fed only by a segment that clips a cell corner that is a
    large *relative* change of a negligible value.  Entries that are zero in
    `want` must be zero in `got`.
    """
    got = np.asarray(got, dtype=np.float64)
    want = np.asarray(want, dtype=np.float64)
    assert got.shape == want.shape
    denom = np.abs(want)
    bad_zero = (denom == 0) & (got != 0)
    assert not bad_zero.any(), f"{bad_zero.sum()} entries nonzero where reference is zero"
    nz = denom > 0
    if not nz.any():
        return 0.0
    floor = scale_floor * float(denom[nz].mean())
    err = np.abs(got[nz] - want[nz]) / (rel * denom[nz] + floor)
    worst = float(err.max())
    assert worst <= 1.0, (f"flux error {worst:.3e} x tolerance (max relative "
                          f"{float((np.abs(got[nz] - want[nz]) / denom[nz]).max()):.3e})")
    return worst


class OracleMonteCarlo:
    """Stands in for MonteCarlo under the command-line driver's loop on the
    CPU (its product path needs a GPU): the same cycles run by the oracle,
    with the reference's observers restated on the oracle's tallies --
    fluence per cell (Tallies.cc:100-118, each group added in order) and the
    census energy spectrum (EnergySpectrum.cc:12-36, the group search of
    NuclearData.cc:207-228)."""

    def __init__(self, deck):
        self.problem = deck.build()
        self.run = oracle_run(self.problem, deck.simulation)
        self.tracker = None
        self.rows = []
        self._fluence = self._spectrum = None

    def observe(self, fluence=False, spectrum=False):
        G = self.problem.num_groups
        self._fluence = np.zeros(self.problem.num_cells) if fluence else None
        self._spectrum = np.zeros(G + 1, dtype=np.uint64) if spectrum else None

    def cycle_init(self):
        self.run.cycle_init()

    def cycle_tracking(self):
        self.run.cycle_tracking(8)
        flux = self.run.flux()
        self.flux_total = flux.sum()
        if self._fluence is not None:
            for g in range(flux.shape[1]):
                self._fluence += flux[:, g]
        if self._spectrum is not None:
            en = self.problem.array("energies")
            G = self.problem.num_groups
            e = self.run.processed()["kinetic_energy"]
            grp = np.minimum(np.searchsorted(en, e, side="right") - 1, G - 1)
            grp[e <= en[0]] = 0
            grp[e > en[-1]] = G
            np.add.at(self._spectrum, grp, 1)

    def cycle_finalize(self):
        self.run.cycle_finalize()
        self.rows.append((self.run.last_balance(), self.flux_total))

    def history(self, first, n):
        from quicksilver_gb300.monte_carlo import CycleHistory
        rows = self.rows[first:first + n]
        return CycleHistory(np.array([r[0] for r in rows]), np.array([r[1] for r in rows]))

    def fluence(self):
        return self._fluence

    def energy_spectrum(self):
        return [self._spectrum]

    def device_status(self):
        return 0

    def close(self):
        pass


def balance_identities(bal: np.ndarray, label: str = "") -> None:
    """The identities the reference's balance counters satisfy every cycle
    (bal [cycles, 13], QSG_BAL_* order): particles tracked = particles ended
    (the reference's own particle-conservation check, CoralBenchmark.cc:152-174,
    and its test for done, MC_Particle_Buffer.cc:176-188), collisions = their
    three kinds (CollisionEvent.cc:103-116), end = census, and each cycle
    starts with the previous cycle's census."""
    from quicksilver_gb300 import _native as N
    b = {k: bal[:, i].astype(np.int64) for k, i in N.BAL.items()}
    np.testing.assert_array_equal(b["start"] + b["source"] + b["split"] - b["rr"] + b["produce"],
                                  b["absorb"] + b["escape"] + b["census"] + b["fission"], err_msg=label)
    np.testing.assert_array_equal(b["collision"], b["scatter"] + b["absorb"] + b["fission"], err_msg=label)
    np.testing.assert_array_equal(b["end"], b["census"], err_msg=label)
    np.testing.assert_array_equal(b["start"][1:], b["census"][:-1], err_msg=label)
