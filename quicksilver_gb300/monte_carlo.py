"""Host mirror of the reference's cycle driver.

``MonteCarlo`` plays the part of Quicksilver's MonteCarlo object plus
main.cc's cycle loop (main.cc:38-85): ``cycle_init`` / ``cycle_tracking`` /
``cycle_finalize`` have the meaning of cycleInit / cycleTracking /
cycleFinalize (main.cc:96-121, 138-307, 310-324), but every step runs on the
GPU through libqsg.so; the host only enqueues work.  ``run`` executes cycles
and returns the per-cycle balance counters and scalar-flux totals, the numbers
the reference prints each cycle (Tallies.cc:123-144).

``BatchMonteCarlo`` runs many independent decks together: one persistent
tracking launch per pass covers every problem, and ``run(use_graph=True)``
replays each whole cycle from a captured CUDA graph.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _native as N
from .problem import Deck, HostProblem
from .tracker import Tracker


@dataclass
class CycleHistory:
    balance: np.ndarray      # [cycles, 13] (single) or [cycles, problems, 13] uint64, BALANCE_FIELDS order
    flux_total: np.ndarray   # [cycles] or [cycles, problems] float64

    def segments(self) -> int:
        return int(self.balance[..., N.BAL["num_segments"]].sum())


def _stream_ptr(stream) -> C.c_void_p:
    """Accept None, a raw cudaStream_t address, or a torch.cuda.Stream."""
    if stream is None:
        return C.c_void_p(0)
    if hasattr(stream, "cuda_stream"):
        return C.c_void_p(stream.cuda_stream)
    return C.c_void_p(int(stream))


def seed_offset(seed: int) -> int:
    """A 64-bit offset derived from a deck's `seed`, for batches that want
    distinct random streams per problem (the reference itself never uses
    `seed`: its source seeds come from cell ids, MC_SourceNow.cc:90-97)."""
    z = (int(seed) + 0x9E3779B97F4A7C15) & 0xFFFFFFFFFFFFFFFF
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & 0xFFFFFFFFFFFFFFFF
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & 0xFFFFFFFFFFFFFFFF
    return z ^ (z >> 31)


class _Driver:
    def _configure(self, decks, problems, store_capacity, seed_offsets):
        sims = [d.simulation for d in decks]
        self._rates = [np.ascontiguousarray(p.source_rates()) for p in problems]
        cfgs = (N.QsgCycleConfig * len(decks))()
        for k, (s, r) in enumerate(zip(sims, self._rates)):
            cfgs[k] = N.QsgCycleConfig(source_rate=r.ctypes.data_as(C.POINTER(C.c_double)), n_particles=s.n_particles,
                                       e_min=s.e_min, e_max=s.e_max, low_weight_cutoff=s.low_weight_cutoff,
                                       load_balance=s.load_balance, reserved=0, store_capacity=store_capacity)
        offs = None
        if seed_offsets is not None:
            self._offs = np.ascontiguousarray(seed_offsets, dtype=np.uint64)
            offs = self._offs.ctypes.data_as(C.POINTER(C.c_uint64))
        N.check(N.lib().qsg_configure_cycle_batch(self.tracker.handle, cfgs, offs))
        self.cycles = 0

    def cycle_init(self, stream=None) -> None:
        N.check(N.lib().qsg_cycle_init(self.tracker.handle, _stream_ptr(stream)))

    def cycle_tracking(self, stream=None) -> None:
        N.check(N.lib().qsg_track_cycle(self.tracker.handle, _stream_ptr(stream)))

    def cycle_finalize(self, stream=None) -> None:
        N.check(N.lib().qsg_cycle_finalize(self.tracker.handle, _stream_ptr(stream)))
        self.cycles += 1

    def _history(self, first, n, problems):
        n = self.cycles - first if n is None else n
        bal = np.zeros((max(n, 0), problems, 13), dtype=np.uint64)
        tot = np.zeros((max(n, 0), problems), dtype=np.float64)
        N.check(N.lib().qsg_cycle_history(self.tracker.handle, first, n,
                                          bal.ctypes.data_as(C.POINTER(C.c_uint64)),
                                          tot.ctypes.data_as(C.POINTER(C.c_double))))
        return bal, tot

    def processing(self) -> np.ndarray:
        """Host copy of the processing store (the particles a cycle will track)."""
        n, _ = self.tracker.sizes()
        cols = N.empty_columns(n)
        soa = N.soa_from_columns(cols)
        got = C.c_uint64()
        N.check(N.lib().qsg_get_processing(self.tracker.handle, C.byref(soa), n, C.byref(got)))
        return N.records_from_columns(cols, got.value)

    def device_status(self, clear: bool = True) -> int:
        return self.tracker.device_status(clear)

    # ---- observability (quicksilver_gb300.observe) ----
    def observe(self, fluence: bool = False, spectrum: bool = False) -> None:
        """Keep the per-cell fluence and / or the census energy spectrum on
        the device from the next finalised cycle on (both start at zero)."""
        flags = (N.QSG_OBSERVE_FLUENCE if fluence else 0) | (N.QSG_OBSERVE_SPECTRUM if spectrum else 0)
        N.check(N.lib().qsg_set_observers(self.tracker.handle, flags))
        self._observe_flags = flags

    def exponential_tally(self, enabled: bool = True) -> None:
        """Run as the reference built with -DEXPONENTIAL_TALLY: one extra
        random number per segment, exp of it tallied per cell (every later
        result then follows that build).  The tally of the running cycle is
        ``cell_tally()``; cycle finalize resets it."""
        self.tracker.set_exponential_tally(enabled)

    def cell_tally(self) -> np.ndarray:
        return self.tracker.cell_tally()

    def fluence(self) -> np.ndarray:
        out = np.zeros(self.tracker.num_cells, dtype=np.float64)
        N.check(N.lib().qsg_read_observers(self.tracker.handle, out.ctypes.data_as(C.POINTER(C.c_double)), None))
        return out

    def energy_spectrum(self) -> np.ndarray:
        """[problems, G+1] census energy-group counts (summed over cycles)."""
        out = np.zeros((len(self.tracker.problems), self.tracker.num_groups + 1), dtype=np.uint64)
        N.check(N.lib().qsg_read_observers(self.tracker.handle, None, out.ctypes.data_as(C.POINTER(C.c_uint64))))
        return out

    def run_cycles(self, n_cycles: int, use_graph: bool = False, stream=None) -> None:
        """n whole cycles enqueued without host synchronisation: each cycle is
        init + QsgOptions.max_passes tracking passes + finalize, replayed from a
        captured CUDA graph when use_graph is set."""
        N.check(N.lib().qsg_run_cycles(self.tracker.handle, n_cycles, int(use_graph), _stream_ptr(stream)))
        self.cycles += n_cycles

    def tune(self, block_size: int = 0, collision_batch: int = 0, queue_chunk: int = 0,
             pool_collision_step: int = 0, pool_refill: int = 0) -> None:
        """Kernel shape (0 keeps a value): threads per block; for the
        one-history-per-lane kernel the collisions batched per warp step and the
        particles claimed per queue atomic; for the pool kernel (default) the
        pooled collisions that make a collision step and the empty slots that
        trigger a refill."""
        N.check(N.lib().qsg_set_tuning(self.tracker.handle, block_size, collision_batch, queue_chunk))
        N.check(N.lib().qsg_set_pool_tuning(self.tracker.handle, pool_collision_step, pool_refill))

    def close(self):
        self.tracker.close()


class MonteCarlo(_Driver):
    def __init__(self, deck: Deck, flux_replicas: int | None = None, balance_replicas: int | None = None,
                 max_passes: int = 8, store_capacity: int = 0, device: int = 0, problem: HostProblem | None = None,
                 block_size: int = 0, collision_batch: int = 0, seed_offset: int = 0):
        """flux_replicas / balance_replicas default to the deck's fTally /
        bTally, the reference's tally replication counts (Tallies.cc:173-238).
        seed_offset (0 = the reference's seeding) is added to every source
        seed, giving an independent replica of the same problem."""
        self.deck = deck
        self.params = deck.simulation
        if flux_replicas is None:
            flux_replicas = max(1, self.params.flux_replications)
        if balance_replicas is None:
            balance_replicas = max(1, self.params.balance_replications)
        self.problem = problem if problem is not None else deck.build()
        self.tracker = Tracker(self.problem, flux_replicas=flux_replicas, balance_replicas=balance_replicas,
                               device=device, max_passes=max_passes, block_size=block_size,
                               collision_batch=collision_batch)
        self._configure([deck], [self.problem], store_capacity, [seed_offset] if seed_offset else None)

    @property
    def n_steps(self) -> int:
        return self.params.n_steps

    def history(self, first: int = 0, n: int | None = None) -> CycleHistory:
        bal, tot = self._history(first, n, 1)
        return CycleHistory(bal[:, 0, :], tot[:, 0])

    def run(self, n_steps: int | None = None, stream=None) -> CycleHistory:
        first = self.cycles
        for _ in range(self.n_steps if n_steps is None else n_steps):
            self.cycle_init(stream)
            self.cycle_tracking(stream)
            self.cycle_finalize(stream)
        hist = self.history(first)
        flags = self.device_status()
        if flags:
            raise N.QsgError(N.QSG_ERR_DEVICE, f"device flags 0x{flags:x} raised during the run")
        return hist


class BatchMonteCarlo(_Driver):
    """Independent decks tracked together (they must share eMin, eMax, nGroups and dt)."""

    def __init__(self, decks: list, flux_replicas: int = 1, balance_replicas: int = 1, max_passes: int = 8,
                 store_capacity: int = 0, device: int = 0, problems: list | None = None,
                 seed_offsets=None, block_size: int = 0, collision_batch: int = 0):
        self.decks = list(decks)
        self.problems = problems if problems is not None else [d.build() for d in self.decks]
        self.tracker = Tracker(self.problems, flux_replicas=flux_replicas, balance_replicas=balance_replicas,
                               device=device, max_passes=max_passes, block_size=block_size,
                               collision_batch=collision_batch)
        self._configure(self.decks, self.problems, store_capacity, seed_offsets)

    @property
    def num_problems(self) -> int:
        return len(self.problems)

    def history(self, first: int = 0, n: int | None = None) -> CycleHistory:
        bal, tot = self._history(first, n, self.num_problems)
        return CycleHistory(bal, tot)

    def run(self, n_cycles: int, use_graph: bool = True, stream=None) -> CycleHistory:
        first = self.cycles
        self.run_cycles(n_cycles, use_graph, stream)
        hist = self.history(first)
        flags = self.device_status()
        if flags:
            raise N.QsgError(N.QSG_ERR_DEVICE, f"device flags 0x{flags:x} raised during the run")
        return hist

