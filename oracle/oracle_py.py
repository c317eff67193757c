"""TEST INFRASTRUCTURE ONLY: ctypes binding of the C oracle (qs_oracle.c).

Used by tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg as
the checker.  Builds ``oracle/_build/libqs_oracle.so`` on first use with the
recipe in ``oracle/Makefile``.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

ORACLE_DIR = Path(__file__).resolve().parent
LIB_PATH = ORACLE_DIR / "_build" / "libqs_oracle.so"

# same 136-byte record as MC_Base_Particle / quicksilver_gb300._native.PARTICLE_DTYPE
PARTICLE_DTYPE = np.dtype([
    ("x", "<f8"), ("y", "<f8"), ("z", "<f8"), ("vx", "<f8"), ("vy", "<f8"), ("vz", "<f8"),
    ("kinetic_energy", "<f8"), ("weight", "<f8"), ("time_to_census", "<f8"), ("age", "<f8"),
    ("num_mean_free_paths", "<f8"), ("num_segments", "<f8"),
    ("random_number_seed", "<u8"), ("identifier", "<u8"),
    ("last_event", "<i4"), ("num_collisions", "<i4"), ("breed", "<i4"), ("species", "<i4"),
    ("domain", "<i4"), ("cell", "<i4"),
])

MAX_PARAMS = 32


class OracleSens(C.Structure):
    """Mirror of OracleSens (qs_oracle.h)."""
    _fields_ = [("K", C.c_int32), ("material", C.c_int32 * MAX_PARAMS), ("reaction", C.c_int32 * MAX_PARAMS),
                ("group_lo", C.c_int32 * MAX_PARAMS), ("group_hi", C.c_int32 * MAX_PARAMS),
                ("theta", C.c_double * MAX_PARAMS), ("flux_cell", C.POINTER(C.c_double)),
                ("dflux", C.POINTER(C.c_double)), ("leak", C.POINTER(C.c_double)), ("dleak", C.POINTER(C.c_double))]


def make_sens(params) -> OracleSens:
    """params: sequence of (material, reaction type, group_lo, group_hi, theta)."""
    s = OracleSens()
    s.K = len(params)
    for k, (m, r, lo, hi, th) in enumerate(params):
        s.material[k], s.reaction[k], s.group_lo[k], s.group_hi[k], s.theta[k] = m, r, lo, hi, th
    return s


_lib = None


def build() -> Path:
    srcs = [ORACLE_DIR / "qs_oracle.c", ORACLE_DIR / "qs_oracle.h", ORACLE_DIR.parent / "include" / "qsg.h"]
    if not LIB_PATH.exists() or any(s.stat().st_mtime > LIB_PATH.stat().st_mtime for s in srcs):
        res = subprocess.run(["make", "-C", str(ORACLE_DIR), "port"], capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"oracle build failed:\n{res.stdout}\n{res.stderr}")
    return LIB_PATH


def compiler_version() -> str:
    """First line of the C compiler's version (the port is built by `make -C oracle port` with it)."""
    try:
        out = subprocess.run(["gcc", "--version"], capture_output=True, text=True, timeout=10).stdout
        return out.splitlines()[0].strip() if out else "unknown"
    except (OSError, subprocess.SubprocessError):
        return "unknown"


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        h = C.CDLL(str(LIB_PATH))
        vp = C.c_void_p
        h.oracle_create.argtypes = [vp, C.POINTER(C.c_double), C.c_uint64, C.c_double, C.c_double,
                                    C.c_double, C.c_int]
        h.oracle_create.restype = vp
        h.oracle_destroy.argtypes = [vp]
        h.oracle_set_seed_offset.argtypes = [vp, C.c_uint64]
        h.oracle_set_seed_offset.restype = None
        h.oracle_use_portable_math.argtypes = [C.c_int]
        h.oracle_use_portable_math.restype = None
        h.oracle_pm_eval.argtypes = [vp, C.c_uint64, vp, vp, vp]
        h.oracle_pm_eval.restype = None
        h.oracle_destroy.restype = None
        for name in ("oracle_cycle_init", "oracle_cycle_finalize"):
            getattr(h, name).argtypes = [vp]
            getattr(h, name).restype = C.c_int
        h.oracle_cycle_tracking.argtypes = [vp, C.c_int]
        h.oracle_cycle_tracking.restype = C.c_int
        for name in ("oracle_num_processing", "oracle_num_processed", "oracle_warning_count"):
            getattr(h, name).argtypes = [vp]
            getattr(h, name).restype = C.c_uint64
        for name in ("oracle_processing", "oracle_processed", "oracle_flux"):
            getattr(h, name).argtypes = [vp]
            getattr(h, name).restype = vp
        h.oracle_set_processing.argtypes = [vp, vp, C.c_uint64]
        h.oracle_set_processing.restype = C.c_int
        for name in ("oracle_balance", "oracle_last_balance"):
            getattr(h, name).argtypes = [vp, C.POINTER(C.c_uint64)]
            getattr(h, name).restype = None
        h.oracle_track.argtypes = [vp, vp, C.c_uint64, vp, C.c_uint64, C.POINTER(C.c_uint64),
                                   C.POINTER(C.c_uint64), C.POINTER(C.c_double), C.c_int]
        h.oracle_track.restype = C.c_int
        h.oracle_track_cell_tally.argtypes = [vp, vp, C.c_uint64, vp, C.c_uint64, C.POINTER(C.c_uint64),
                                              C.POINTER(C.c_uint64), C.POINTER(C.c_double), C.POINTER(C.c_double),
                                              C.c_int]
        h.oracle_track_cell_tally.restype = C.c_int
        h.oracle_enable_exponential_tally.argtypes = [vp]
        h.oracle_enable_exponential_tally.restype = C.c_int
        h.oracle_read_cell_tally.argtypes = [vp, vp]
        h.oracle_read_cell_tally.restype = C.c_int
        h.oracle_track_sens.argtypes = [vp, C.POINTER(OracleSens), vp, vp, C.c_uint64, vp, vp, C.c_uint64,
                                        C.POINTER(C.c_uint64), C.POINTER(C.c_uint64), C.POINTER(C.c_double), C.c_int]
        h.oracle_track_sens.restype = C.c_int
        h.oracle_enable_sensitivity.argtypes = [vp, C.POINTER(OracleSens)]
        h.oracle_enable_sensitivity.restype = C.c_int
        h.oracle_read_sensitivity.argtypes = [vp, vp, vp, vp, vp]
        h.oracle_read_sensitivity.restype = C.c_int
        for name in ("oracle_processing_scores", "oracle_processed_scores"):
            getattr(h, name).argtypes = [vp]
            getattr(h, name).restype = vp
        h.oracle_rng_sample.argtypes = [C.POINTER(C.c_uint64)]
        h.oracle_rng_sample.restype = C.c_double
        h.oracle_rng_spawn.argtypes = [C.POINTER(C.c_uint64)]
        h.oracle_rng_spawn.restype = C.c_uint64
        h.oracle_flop_counts.argtypes = [C.POINTER(C.c_uint64)]
        h.oracle_flop_counts.restype = None
        h.oracle_reset_flop_counts.argtypes = []
        h.oracle_reset_flop_counts.restype = None
        _lib = h
    return _lib


class OracleRun:
    """Whole-cycle CPU restatement over a QsgProblem (keeps `keepalive` alive)."""

    def __init__(self, problem_ptr, num_cells: int, num_groups: int, source_rates: np.ndarray,
                 n_particles: int, e_min: float, e_max: float, low_weight_cutoff: float,
                 load_balance: int, keepalive=None):
        self._keep = (keepalive, source_rates)
        self._rates = np.ascontiguousarray(source_rates, dtype=np.float64)
        self.num_cells, self.num_groups = num_cells, num_groups
        self._h = lib().oracle_create(problem_ptr, self._rates.ctypes.data_as(C.POINTER(C.c_double)),
                                      n_particles, e_min, e_max, low_weight_cutoff, load_balance)
        if not self._h:
            raise MemoryError("oracle_create failed")

    def set_seed_offset(self, offset: int):
        """Add `offset` to every source seed (before the first cycle): the
        oracle's side of the library's per-problem seed offsets."""
        lib().oracle_set_seed_offset(self._h, int(offset) & 0xFFFFFFFFFFFFFFFF)

    def close(self):
        if self._h:
            lib().oracle_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def cycle_init(self):
        if lib().oracle_cycle_init(self._h):
            raise RuntimeError("oracle_cycle_init failed")

    def cycle_tracking(self, nthreads: int = 0):
        if lib().oracle_cycle_tracking(self._h, nthreads):
            raise RuntimeError("oracle_cycle_tracking failed")

    def cycle_finalize(self):
        lib().oracle_cycle_finalize(self._h)

    def _particles(self, ptr, n) -> np.ndarray:
        if n == 0:
            return np.empty(0, dtype=PARTICLE_DTYPE)
        buf = (C.c_char * (n * PARTICLE_DTYPE.itemsize)).from_address(ptr)
        return np.frombuffer(buf, dtype=PARTICLE_DTYPE).copy()

    def processing(self) -> np.ndarray:
        return self._particles(lib().oracle_processing(self._h), lib().oracle_num_processing(self._h))

    def processed(self) -> np.ndarray:
        return self._particles(lib().oracle_processed(self._h), lib().oracle_num_processed(self._h))

    def set_processing(self, recs: np.ndarray):
        recs = np.ascontiguousarray(recs, dtype=PARTICLE_DTYPE)
        if lib().oracle_set_processing(self._h, recs.ctypes.data, len(recs)):
            raise MemoryError("oracle_set_processing failed")

    def balance(self) -> np.ndarray:
        out = (C.c_uint64 * 13)()
        lib().oracle_balance(self._h, out)
        return np.array(out, dtype=np.uint64)

    def last_balance(self) -> np.ndarray:
        out = (C.c_uint64 * 13)()
        lib().oracle_last_balance(self._h, out)
        return np.array(out, dtype=np.uint64)

    def flux(self) -> np.ndarray:
        n = self.num_cells * self.num_groups
        buf = (C.c_double * n).from_address(lib().oracle_flux(self._h))
        return np.frombuffer(buf, dtype=np.float64).copy().reshape(self.num_cells, self.num_groups)

    def warnings(self) -> int:
        return int(lib().oracle_warning_count(self._h))

    def enable_exponential_tally(self):
        """Behave as the reference built with -DEXPONENTIAL_TALLY (an extra
        random number per segment, exp of it tallied per cell)."""
        if lib().oracle_enable_exponential_tally(self._h):
            raise RuntimeError("oracle_enable_exponential_tally failed")

    def cell_tally(self) -> np.ndarray:
        """[C] exponential cell tally of the running cycle (reset by cycle_finalize)."""
        out = np.zeros(self.num_cells)
        if lib().oracle_read_cell_tally(self._h, out.ctypes.data):
            raise RuntimeError("exponential cell tally is off")
        return out

    def enable_sensitivity(self, params):
        """params: (material, reaction type, group_lo, group_hi, theta) per parameter."""
        self._sens = make_sens(params)
        if lib().oracle_enable_sensitivity(self._h, C.byref(self._sens)):
            raise RuntimeError("oracle_enable_sensitivity failed (call it before the first cycle)")
        self.K = len(params)

    def read_sensitivity(self):
        """(flux_cell [C], dflux [C, K], leak, dleak [K]) accumulated over all cycles."""
        fc = np.zeros(self.num_cells)
        df = np.zeros(self.num_cells * self.K)
        lk = np.zeros(1)
        dl = np.zeros(self.K)
        if lib().oracle_read_sensitivity(self._h, fc.ctypes.data, df.ctypes.data, lk.ctypes.data, dl.ctypes.data):
            raise RuntimeError("oracle_read_sensitivity failed")
        return fc, df.reshape(self.num_cells, self.K), float(lk[0]), dl

    def processing_scores(self) -> np.ndarray:
        n = lib().oracle_num_processing(self._h)
        if n == 0:
            return np.zeros((0, self.K))
        buf = (C.c_double * (n * self.K)).from_address(lib().oracle_processing_scores(self._h))
        return np.frombuffer(buf, dtype=np.float64).copy().reshape(n, self.K)

    def processed_scores(self) -> np.ndarray:
        n = lib().oracle_num_processed(self._h)
        if n == 0:
            return np.zeros((0, self.K))
        buf = (C.c_double * (n * self.K)).from_address(lib().oracle_processed_scores(self._h))
        return np.frombuffer(buf, dtype=np.float64).copy().reshape(n, self.K)


def track(problem_ptr, num_cells: int, num_groups: int, particles: np.ndarray, nthreads: int = 0,
          cell_tally: bool = False):
    """One-shot tracking: returns (census records, balance[13], flux[C, G]),
    plus the exponential cell tally [C] when ``cell_tally`` (the reference's
    EXPONENTIAL_TALLY build)."""
    recs = np.ascontiguousarray(particles, dtype=PARTICLE_DTYPE)
    n = len(recs)
    cap = max(4 * n + 16, 1024)
    while True:
        census = np.empty(cap, dtype=PARTICLE_DTYPE)
        bal = (C.c_uint64 * 13)()
        flux = np.zeros(num_cells * num_groups, dtype=np.float64)
        ct = np.zeros(num_cells, dtype=np.float64)
        n_census = C.c_uint64(0)
        st = lib().oracle_track_cell_tally(problem_ptr, recs.ctypes.data if n else None, n, census.ctypes.data, cap,
                                           C.byref(n_census), bal, flux.ctypes.data_as(C.POINTER(C.c_double)),
                                           ct.ctypes.data_as(C.POINTER(C.c_double)) if cell_tally else None,
                                           nthreads)
        if st == -3:   # fission grew the population past the census room: again, with room for all
            cap = n_census.value + 16
            continue
        break
    if st:
        raise RuntimeError(f"oracle_track failed ({st})")
    out = (census[: n_census.value].copy(), np.array(bal, dtype=np.uint64), flux.reshape(num_cells, num_groups))
    return out + (ct,) if cell_tally else out


def track_sens(problem_ptr, num_cells: int, num_groups: int, particles: np.ndarray, params, scores=None,
               nthreads: int = 0):
    """One-shot tracking with sensitivity scores.  Returns a dict: census,
    census_scores [n, K], balance[13], flux[C, G], flux_cell [C], dflux [C, K],
    leak, dleak [K]."""
    recs = np.ascontiguousarray(particles, dtype=PARTICLE_DTYPE)
    n = len(recs)
    K = len(params)
    sc_in = None if scores is None else np.ascontiguousarray(scores, dtype=np.float64).reshape(n, K)
    cap = max(4 * n + 16, 1024)
    while True:   # a census larger than cap: run again with room for it (outputs start from zero)
        sens = make_sens(params)
        fc, df, lk, dl = np.zeros(num_cells), np.zeros(num_cells * K), np.zeros(1), np.zeros(K)
        sens.flux_cell = fc.ctypes.data_as(C.POINTER(C.c_double))
        sens.dflux = df.ctypes.data_as(C.POINTER(C.c_double))
        sens.leak = lk.ctypes.data_as(C.POINTER(C.c_double))
        sens.dleak = dl.ctypes.data_as(C.POINTER(C.c_double))
        census = np.empty(cap, dtype=PARTICLE_DTYPE)
        census_sc = np.empty((cap, K))
        bal = (C.c_uint64 * 13)()
        flux = np.zeros(num_cells * num_groups, dtype=np.float64)
        n_census = C.c_uint64(0)
        st = lib().oracle_track_sens(problem_ptr, C.byref(sens), recs.ctypes.data if n else None,
                                     sc_in.ctypes.data if sc_in is not None and n else None, n, census.ctypes.data,
                                     census_sc.ctypes.data, cap, C.byref(n_census), bal,
                                     flux.ctypes.data_as(C.POINTER(C.c_double)), nthreads)
        if st == -3:
            cap = n_census.value + 16
            continue
        if st:
            raise RuntimeError(f"oracle_track_sens failed ({st})")
        break
    m = n_census.value
    return {"census": census[:m].copy(), "census_scores": census_sc[:m].copy(),
            "balance": np.array(bal, dtype=np.uint64), "flux": flux.reshape(num_cells, num_groups),
            "flux_cell": fc, "dflux": df.reshape(num_cells, K), "leak": float(lk[0]), "dleak": dl}


def use_portable_math(on: bool):
    """Process-wide: the tracking path's log / sin / cos become the portable
    functions (quicksilver_gb300/csrc/portable_math.h) or, off, libm's."""
    lib().oracle_use_portable_math(int(bool(on)))


def flop_counts(reset: bool = False):
    """(FP64 operations, elementary-function calls) of the tracking path
    since the last reset, counted as the reference writes them."""
    out = (C.c_uint64 * 2)()
    lib().oracle_flop_counts(out)
    if reset:
        lib().oracle_reset_flop_counts()
    return int(out[0]), int(out[1])


def pm_eval(x: np.ndarray):
    """(log, sin, cos) of x by the portable functions."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = [np.empty_like(x) for _ in range(3)]
    lib().oracle_pm_eval(x.ctypes.data, len(x), *(o.ctypes.data for o in out))
    return tuple(out)


def rng_sample(seed: int):
    s = C.c_uint64(seed)
    v = lib().oracle_rng_sample(C.byref(s))
    return v, s.value


def rng_spawn(seed: int):
    s = C.c_uint64(seed)
    child = lib().oracle_rng_spawn(C.byref(s))
    return child, s.value
