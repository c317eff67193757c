"""Host mirror of the reference's cycle driver.

``MonteCarlo`` plays the part of Quicksilver's MonteCarlo object plus
main.cc's cycle loop (main.cc:38-85): ``cycle_init`` / ``cycle_tracking`` /
``cycle_finalize`` have the meaning of cycleInit / cycleTracking /
cycleFinalize (main.cc:96-121, 138-307, 310-324), but every step runs on the
GPU through libqsg.so; the host only enqueues work.  ``run`` executes
``nSteps`` cycles and returns the per-cycle balance counters and scalar-flux
totals, the numbers the reference prints each cycle (Tallies.cc:123-144).
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
    balance: np.ndarray      # [cycles, 13] uint64, BALANCE_FIELDS order
    flux_total: np.ndarray   # [cycles] float64

    def segments(self) -> int:
        return int(self.balance[:, N.BAL["num_segments"]].sum())


def _stream_ptr(stream) -> C.c_void_p:
    """Accept None, a raw cudaStream_t address, or a torch.cuda.Stream."""
    if stream is None:
        return C.c_void_p(0)
    if hasattr(stream, "cuda_stream"):
        return C.c_void_p(stream.cuda_stream)
    return C.c_void_p(int(stream))


class MonteCarlo:
    def __init__(self, deck: Deck, flux_replicas: int = 1, balance_replicas: int = 1, max_passes: int = 8,
                 store_capacity: int = 0, device: int = 0, problem: HostProblem | None = None):
        self.deck = deck
        self.params = deck.simulation
        self.problem = problem if problem is not None else deck.build()
        self.tracker = Tracker(self.problem, flux_replicas=flux_replicas, balance_replicas=balance_replicas,
                               device=device, max_passes=max_passes)
        self._rates = np.ascontiguousarray(self.problem.source_rates())
        cfg = N.QsgCycleConfig(source_rate=self._rates.ctypes.data_as(C.POINTER(C.c_double)),
                               n_particles=self.params.n_particles, e_min=self.params.e_min,
                               e_max=self.params.e_max, low_weight_cutoff=self.params.low_weight_cutoff,
                               load_balance=self.params.load_balance, reserved=0, store_capacity=store_capacity)
        N.check(N.lib().qsg_configure_cycle(self.tracker.handle, C.byref(cfg)))
        self.cycles = 0

    @property
    def n_steps(self) -> int:
        return self.params.n_steps

    def cycle_init(self, stream=None) -> None:
        N.check(N.lib().qsg_cycle_init(self.tracker.handle, _stream_ptr(stream)))

    def cycle_tracking(self, stream=None) -> None:
        N.check(N.lib().qsg_track_cycle(self.tracker.handle, _stream_ptr(stream)))

    def cycle_finalize(self, stream=None) -> None:
        N.check(N.lib().qsg_cycle_finalize(self.tracker.handle, _stream_ptr(stream)))
        self.cycles += 1

    def history(self, first: int = 0, n: int | None = None) -> CycleHistory:
        n = self.cycles - first if n is None else n
        bal = np.zeros((max(n, 0), 13), dtype=np.uint64)
        tot = np.zeros(max(n, 0), dtype=np.float64)
        N.check(N.lib().qsg_cycle_history(self.tracker.handle, first, n,
                                          bal.ctypes.data_as(C.POINTER(C.c_uint64)),
                                          tot.ctypes.data_as(C.POINTER(C.c_double))))
        return CycleHistory(bal, tot)

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

    def close(self):
        self.tracker.close()
