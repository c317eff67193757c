"""Python face of the C-ABI tracking handle (libqsg.so, include/qsg.h).

``Tracker`` is the drop-in for the per-vault tracking launch of the
reference's ``cycleTracking`` (main.cc:155-236): upload the processing
particles, track them on the GPU, read back census particles and tallies.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N
from .problem import HostProblem


class Tracker:
    def __init__(self, problem: HostProblem | list, flux_replicas: int = 1, balance_replicas: int = 1,
                 particle_capacity: int = 0, max_segments: int = 0, device: int = 0, max_passes: int = 0,
                 block_size: int = 0, collision_batch: int = 0):
        """One problem, or a list of problems tracked together as a batch
        (qsg_batch_create: they must share the energy grid and time step)."""
        opts = N.QsgOptions(device=device, block_size=block_size, flux_replicas=flux_replicas,
                            balance_replicas=balance_replicas, particle_capacity=particle_capacity,
                            max_segments=max_segments, max_passes=max_passes, collision_batch=collision_batch)
        self._h = C.c_void_p()
        if isinstance(problem, (list, tuple)):
            self.problems = list(problem)
            views = (N.QsgProblem * len(self.problems))(*[p.view for p in self.problems])
            N.check(N.lib().qsg_batch_create(views, len(self.problems), C.byref(opts), C.byref(self._h)))
            self.problem = self.problems[0]
        else:
            self.problems = [problem]
            self.problem = problem
            N.check(N.lib().qsg_create(C.byref(problem.view), C.byref(opts), C.byref(self._h)))
        n = C.c_int32()
        offs = np.zeros(len(self.problems) + 1, dtype=np.int32)
        N.check(N.lib().qsg_num_problems(self._h, C.byref(n), offs.ctypes.data_as(C.POINTER(C.c_int32))))
        self.cell_offsets = offs
        self.num_cells = int(offs[-1])
        self.num_groups = self.problem.num_groups

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    def close(self):
        if self._h:
            N.lib().qsg_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_particles(self, records: np.ndarray) -> None:
        recs = np.ascontiguousarray(records, dtype=N.PARTICLE_DTYPE)
        cols = N.columns_of(recs)
        soa = N.soa_from_columns(cols)
        N.check(N.lib().qsg_set_particles(self._h, C.byref(soa), len(recs)))

    def set_track_kernel(self, kind: int) -> None:
        """1 (default): warp particle pools; 0: one history per lane."""
        N.check(N.lib().qsg_set_track_kernel(self._h, kind))

    def track(self) -> None:
        N.check(N.lib().qsg_track_cycle_sync(self._h))

    def track_host(self, inputs: dict, n: int, census: dict, capacity: int, stream=None) -> int:
        """qsg_track_host: track the ``n`` particles in ``inputs`` and append
        census particles to ``census`` (room for ``capacity``), both mapping
        SoA field names to page-locked host arrays (torch tensors made with
        ``pin_memory=True``, or numpy views of page-locked memory); the GPU
        reads and writes them over the host link during tracking.  Returns
        the census count; tallies accumulate in the handle."""
        def ptr(a):
            return a.data_ptr() if hasattr(a, "data_ptr") else a.ctypes.data
        si = N.soa_from_pointers({k: ptr(v) for k, v in inputs.items()})
        so = N.soa_from_pointers({k: ptr(v) for k, v in census.items()})
        got = C.c_uint64()
        N.check(N.lib().qsg_track_host(self._h, C.byref(si), n, C.byref(so), capacity, C.byref(got),
                                       C.c_void_p(stream) if stream else None))
        return got.value

    def sizes(self):
        a, b = C.c_uint64(), C.c_uint64()
        N.check(N.lib().qsg_sizes(self._h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def census(self) -> np.ndarray:
        _, n = self.sizes()
        cols = N.empty_columns(n)
        soa = N.soa_from_columns(cols)
        got = C.c_uint64()
        N.check(N.lib().qsg_get_census(self._h, C.byref(soa), n, C.byref(got)))
        return N.records_from_columns(cols, got.value)

    def tallies(self):
        bal = np.zeros(13, dtype=np.uint64)
        flux = np.zeros(self.num_cells * self.num_groups, dtype=np.float64)
        N.check(N.lib().qsg_read_tallies(self._h, bal.ctypes.data_as(C.POINTER(C.c_uint64)),
                                         flux.ctypes.data_as(C.POINTER(C.c_double))))
        return bal, flux.reshape(self.num_cells, self.num_groups)

    def reset_tallies(self) -> None:
        N.check(N.lib().qsg_reset_tallies(self._h))

    def set_exponential_tally(self, enabled: bool = True) -> None:
        """qsg_set_exponential_tally: the reference's -DEXPONENTIAL_TALLY build."""
        N.check(N.lib().qsg_set_exponential_tally(self._h, int(enabled)))

    def cell_tally(self) -> np.ndarray:
        """[num_cells] exponential cell tally since the last reset."""
        out = np.zeros(self.num_cells, dtype=np.float64)
        N.check(N.lib().qsg_read_cell_tally(self._h, out.ctypes.data_as(C.POINTER(C.c_double))))
        return out

    # ---- sensitivities (qsg_enable_sensitivity) ----
    def material_offsets(self) -> np.ndarray:
        """[problems + 1] offsets of each problem's materials in this handle."""
        out = np.zeros(len(self.problems) + 1, dtype=np.int32)
        N.check(N.lib().qsg_material_offsets(self._h, out.ctypes.data_as(C.POINTER(C.c_int32))))
        return out

    def enable_sensitivity(self, params) -> None:
        """params: sequence of sensitivity.Param (material indices of this handle)."""
        rows = [(k, *e) for k, p in enumerate(params) for e in p.entries()]
        cols = [np.ascontiguousarray([r[j] for r in rows], dtype=np.int32) for j in range(5)]
        theta = np.ascontiguousarray([p.theta for p in params], dtype=np.float64)
        ip = C.POINTER(C.c_int32)
        s = N.QsgSensitivity(len(params), theta.ctypes.data_as(C.POINTER(C.c_double)), len(rows),
                             *(c.ctypes.data_as(ip) for c in cols))
        N.check(N.lib().qsg_enable_sensitivity(self._h, C.byref(s)))
        self.num_params = len(params)

    def read_sensitivity(self) -> dict:
        """flux_cell [C], dflux [C, K], leak [P], dleak [P, K] accumulated since enable / reset."""
        K, P = self.num_params, len(self.problems)
        out = {"flux_cell": np.zeros(self.num_cells), "dflux": np.zeros((self.num_cells, K)),
               "leak": np.zeros(P), "dleak": np.zeros((P, K))}
        dp = C.POINTER(C.c_double)
        N.check(N.lib().qsg_read_sensitivity(self._h, *(out[k].ctypes.data_as(dp)
                                                       for k in ("flux_cell", "dflux", "leak", "dleak"))))
        return out

    def reset_sensitivity(self) -> None:
        N.check(N.lib().qsg_reset_sensitivity(self._h))

    def device_status(self, clear: bool = True) -> int:
        f = C.c_uint32()
        N.check(N.lib().qsg_device_status(self._h, C.byref(f), int(clear)))
        return f.value
