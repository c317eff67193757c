"""ctypes binding of libqsg.so (declarations mirror include/qsg.h).

The library is built in-tree by :mod:`quicksilver_gb300.build`.  Loading it
needs no GPU; every tracking entry point fails with QSG_ERR_NO_DEVICE when no
CUDA device is visible -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

import os

# QSG_LIB=<name> loads lib/libqsg_<name>.so instead of lib/libqsg.so, e.g.
# QSG_LIB=verify for the screen-verification build (build.py --verify-screen),
# QSG_LIB=nvtx for the build with NVTX ranges (build.py --nvtx)
_variant = os.environ.get("QSG_LIB", "")
LIB_PATH = Path(__file__).resolve().parent / "lib" / (f"libqsg_{_variant}.so" if _variant else "libqsg.so")

QSG_OK = 0
QSG_ERR_INVALID = 1
QSG_ERR_CUDA = 2
QSG_ERR_CAPACITY = 3
QSG_ERR_DEVICE = 4
QSG_ERR_UNSUPPORTED = 5
QSG_ERR_IO = 6
QSG_ERR_NO_DEVICE = 7
QSG_OBSERVE_FLUENCE = 1
QSG_OBSERVE_SPECTRUM = 2
# device error flag bits (qsg_device_status)
QSG_DEV_SEGMENT_LIMIT = 1 << 0
QSG_DEV_TRACKING_LIMIT = 1 << 1
QSG_DEV_NO_REACTION = 1 << 2
QSG_DEV_OFF_PROCESSOR = 1 << 3
QSG_DEV_STORE_OVERFLOW = 1 << 4
QSG_DEV_BAD_FACET = 1 << 5
QSG_DEV_NEGATIVE_DISTANCE = 1 << 6
QSG_DEV_PASS_LIMIT = 1 << 7
QSG_DEV_SCREEN_MISS = 1 << 8   # verification build only

# NuclearDataReaction::Enum (NuclearData.hh:33-40), QSG_REACT_* in qsg.h
QSG_REACT_SCATTER, QSG_REACT_ABSORPTION, QSG_REACT_FISSION = 1, 2, 3

BALANCE_FIELDS = ("absorb", "census", "escape", "collision", "end", "fission", "produce",
                  "scatter", "start", "source", "rr", "split", "num_segments")
BAL = {name: i for i, name in enumerate(BALANCE_FIELDS)}

# MC_Base_Particle field order (MC_Base_Particle.hh:75-92), 136 bytes.
PARTICLE_DTYPE = np.dtype([
    ("x", "<f8"), ("y", "<f8"), ("z", "<f8"), ("vx", "<f8"), ("vy", "<f8"), ("vz", "<f8"),
    ("kinetic_energy", "<f8"), ("weight", "<f8"), ("time_to_census", "<f8"), ("age", "<f8"),
    ("num_mean_free_paths", "<f8"), ("num_segments", "<f8"),
    ("random_number_seed", "<u8"), ("identifier", "<u8"),
    ("last_event", "<i4"), ("num_collisions", "<i4"), ("breed", "<i4"), ("species", "<i4"),
    ("domain", "<i4"), ("cell", "<i4"),
])
assert PARTICLE_DTYPE.itemsize == 136
SOA_FIELDS = PARTICLE_DTYPE.names

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)
_up = C.POINTER(C.c_uint64)


class QsgProblem(C.Structure):
    _fields_ = [
        ("num_groups", C.c_int32), ("energies", _dp),
        ("num_isotopes", C.c_int32), ("isotope_reaction_offset", _ip), ("reaction_type", _ip),
        ("reaction_nubar", _dp), ("reaction_xs", _dp),
        ("num_materials", C.c_int32), ("material_isotope_offset", _ip), ("material_isotope_gid", _ip),
        ("material_atom_fraction", _dp), ("material_mass", _dp),
        ("num_cells", C.c_int32), ("num_nodes", C.c_int32), ("nodes", _dp), ("cell_points", _ip),
        ("facet_local_points", _ip), ("facet_planes", _dp), ("facet_event", _ip),
        ("facet_adjacent_cell", _ip), ("facet_adjacent_facet", _ip), ("cell_material", _ip),
        ("cell_number_density", _dp), ("cell_volume", _dp), ("cell_id", _up),
        ("time_step", C.c_double),
    ]


class QsgParticleSoA(C.Structure):
    _fields_ = [(name, _dp) for name in SOA_FIELDS[:12]] + \
               [(name, _up) for name in SOA_FIELDS[12:14]] + \
               [(name, _ip) for name in SOA_FIELDS[14:]]


class QsgOptions(C.Structure):
    _fields_ = [("device", C.c_int32), ("block_size", C.c_int32), ("flux_replicas", C.c_int32),
                ("balance_replicas", C.c_int32), ("particle_capacity", C.c_uint64),
                ("max_segments", C.c_uint64), ("max_passes", C.c_int32), ("collision_batch", C.c_int32)]


class QsgSimulation(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("dt", "lx", "ly", "lz", "e_min", "e_max", "low_weight_cutoff")] + \
               [(n, C.c_uint64) for n in ("n_particles", "batch_size", "n_batches")] + \
               [(n, C.c_int32) for n in ("n_steps", "nx", "ny", "nz", "seed", "x_dom", "y_dom", "z_dom",
                                         "n_groups", "load_balance", "balance_replications",
                                         "flux_replications", "cell_replications", "coral_benchmark",
                                         "boundary_condition")]


class QsgCycleConfig(C.Structure):
    _fields_ = [("source_rate", _dp), ("n_particles", C.c_uint64), ("e_min", C.c_double), ("e_max", C.c_double),
                ("low_weight_cutoff", C.c_double), ("load_balance", C.c_int32), ("reserved", C.c_int32),
                ("store_capacity", C.c_uint64)]


MAX_PARAMS = 32


class QsgSensitivity(C.Structure):
    _fields_ = [("num_params", C.c_int32), ("theta", C.POINTER(C.c_double)), ("num_entries", C.c_int32),
                ("param", C.POINTER(C.c_int32)), ("material", C.POINTER(C.c_int32)),
                ("reaction", C.POINTER(C.c_int32)), ("group_lo", C.POINTER(C.c_int32)),
                ("group_hi", C.POINTER(C.c_int32))]


class QsgError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"qsg error {code}: {message}")
        self.code = code


_lib = None
_VP = C.c_void_p

_SIGNATURES = {
    "qsg_abi_version": ([], C.c_int),
    "qsg_last_error": ([C.c_char_p, C.c_size_t], C.c_int),
    "qsg_device_count": ([C.POINTER(C.c_int)], C.c_int),
    "qsg_problem_check": ([C.POINTER(QsgProblem)], C.c_int),
    "qsg_check_arithmetic": ([C.c_int32, C.c_uint64, C.c_uint64, C.POINTER(C.c_uint64)], C.c_int),
    "qsg_measure_fp64_rate": ([C.c_int32, C.POINTER(C.c_double)], C.c_int),
    "qsg_portable_math_eval": ([C.c_int32, _VP, C.c_uint64, _VP, _VP, _VP], C.c_int),
    "qsg_create": ([C.POINTER(QsgProblem), C.POINTER(QsgOptions), C.POINTER(_VP)], C.c_int),
    "qsg_destroy": ([_VP], C.c_int),
    "qsg_set_particles": ([_VP, C.POINTER(QsgParticleSoA), C.c_uint64], C.c_int),
    "qsg_begin_cycle_from_census": ([_VP, C.POINTER(C.c_uint64)], C.c_int),
    "qsg_sizes": ([_VP, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)], C.c_int),
    "qsg_get_census": ([_VP, C.POINTER(QsgParticleSoA), C.c_uint64, C.POINTER(C.c_uint64)], C.c_int),
    "qsg_track_cycle": ([_VP, _VP], C.c_int),
    "qsg_track_cycle_sync": ([_VP], C.c_int),
    "qsg_track_cycle_async": ([_VP, _VP], C.c_int),
    "qsg_track_particles_noalloc": ([_VP, C.POINTER(QsgParticleSoA), C.c_uint64, C.POINTER(QsgParticleSoA), C.c_uint64,
                                     C.POINTER(C.c_uint64), _VP, _VP, _VP], C.c_int),
    "qsg_track_host": ([_VP, C.POINTER(QsgParticleSoA), C.c_uint64, C.POINTER(QsgParticleSoA), C.c_uint64,
                        C.POINTER(C.c_uint64), _VP], C.c_int),
    "qsg_set_exponential_tally": ([_VP, C.c_int32], C.c_int),
    "qsg_read_cell_tally": ([_VP, _dp], C.c_int),
    "qsg_read_tallies": ([_VP, _up, _dp], C.c_int),
    "qsg_reset_tallies": ([_VP], C.c_int),
    "qsg_device_status": ([_VP, C.POINTER(C.c_uint32), C.c_int], C.c_int),
    "qsg_configure_cycle": ([_VP, C.POINTER(QsgCycleConfig)], C.c_int),
    "qsg_configure_cycle_batch": ([_VP, C.POINTER(QsgCycleConfig), _up], C.c_int),
    "qsg_batch_create": ([C.POINTER(QsgProblem), C.c_int32, C.POINTER(QsgOptions), C.POINTER(_VP)], C.c_int),
    "qsg_num_problems": ([_VP, C.POINTER(C.c_int32), _ip], C.c_int),
    "qsg_set_tuning": ([_VP, C.c_int32, C.c_int32, C.c_int32], C.c_int),
    "qsg_set_track_kernel": ([_VP, C.c_int32], C.c_int),
    "qsg_set_pool_tuning": ([_VP, C.c_int32, C.c_int32], C.c_int),
    "qsg_run_cycles": ([_VP, C.c_int32, C.c_int32, _VP], C.c_int),
    "qsg_cycle_init": ([_VP, _VP], C.c_int),
    "qsg_cycle_finalize": ([_VP, _VP], C.c_int),
    "qsg_cycle_history": ([_VP, C.c_uint64, C.c_uint64, _up, _dp], C.c_int),
    "qsg_get_processing": ([_VP, C.POINTER(QsgParticleSoA), C.c_uint64, C.POINTER(C.c_uint64)], C.c_int),
    "qsg_processing_view": ([_VP, C.POINTER(QsgParticleSoA), C.POINTER(C.c_uint64)], C.c_int),
    "qsg_enable_sensitivity": ([_VP, C.POINTER(QsgSensitivity)], C.c_int),
    "qsg_read_sensitivity": ([_VP, _dp, _dp, _dp, _dp], C.c_int),
    "qsg_reset_sensitivity": ([_VP], C.c_int),
    "qsg_material_offsets": ([_VP, _ip], C.c_int),
    "qsg_processed_view": ([_VP, C.POINTER(QsgParticleSoA), C.POINTER(C.c_uint64)], C.c_int),
    "qsg_deck_parse_file": ([C.c_char_p, C.POINTER(_VP)], C.c_int),
    "qsg_deck_parse_string": ([C.c_char_p, C.POINTER(_VP)], C.c_int),
    "qsg_deck_set": ([_VP, C.c_char_p, C.c_char_p], C.c_int),
    "qsg_deck_free": ([_VP], C.c_int),
    "qsg_deck_simulation": ([_VP, C.POINTER(QsgSimulation)], C.c_int),
    "qsg_deck_energy_spectrum": ([_VP, C.c_char_p, C.c_size_t], C.c_int),
    "qsg_deck_write": ([_VP, C.c_char_p, C.c_size_t, C.POINTER(C.c_size_t)], C.c_int),
    "qsg_set_observers": ([_VP, C.c_int32], C.c_int),
    "qsg_read_observers": ([_VP, _dp, _up], C.c_int),
    "qsg_deck_build": ([_VP, C.POINTER(_VP)], C.c_int),
    "qsg_host_problem_view": ([_VP, C.POINTER(QsgProblem)], C.c_int),
    "qsg_host_problem_source_rates": ([_VP, _dp, C.c_int32], C.c_int),
    "qsg_host_problem_scale_xs": ([_VP, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_double], C.c_int),
    "qsg_host_problem_free": ([_VP], C.c_int),
}


def lib() -> C.CDLL:
    """Load libqsg.so (building it first if it is missing)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            from . import build as _build
            _build.build(verify_screen=LIB_PATH.name == "libqsg_verify.so", nvtx=LIB_PATH.name == "libqsg_nvtx.so")
        handle = C.CDLL(str(LIB_PATH))
        for name, (args, res) in _SIGNATURES.items():
            fn = getattr(handle, name)
            fn.argtypes = args
            fn.restype = res
        _lib = handle
    return _lib


def last_error() -> str:
    buf = C.create_string_buffer(2048)
    lib().qsg_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


def check(code: int) -> None:
    if code != QSG_OK:
        raise QsgError(code, last_error())


def device_count() -> int:
    n = C.c_int(0)
    check(lib().qsg_device_count(C.byref(n)))
    return n.value


def check_arithmetic(n: int, seed: int = 1, device: int = 0) -> tuple:
    """Disagreements (conversion, quotient, comparisons, random-number sample)
    of the tracking loop's replacements of FP64 operations with those
    operations, on ``n`` random operands per kind (qsg_check_arithmetic)."""
    out = (C.c_uint64 * 4)()
    check(lib().qsg_check_arithmetic(device, n, seed, out))
    return tuple(int(v) for v in out)


def portable_math_eval(x, device: int = 0):
    """(log, sin, cos) of x by the portable elementary functions on the GPU
    (qsg_portable_math_eval)."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = [np.empty_like(x) for _ in range(3)]
    check(lib().qsg_portable_math_eval(device, x.ctypes.data, len(x), *(o.ctypes.data for o in out)))
    return tuple(out)


def measure_fp64_rate(device: int = 0) -> float:
    """FP64 warp instructions per second the device issues (qsg_measure_fp64_rate)."""
    out = C.c_double(0.0)
    check(lib().qsg_measure_fp64_rate(device, C.byref(out)))
    return out.value


def soa_from_columns(cols: dict) -> QsgParticleSoA:
    """Build a QsgParticleSoA view over contiguous numpy columns (kept alive by the caller)."""
    soa = QsgParticleSoA()
    for name in SOA_FIELDS:
        arr = cols[name]
        assert arr.flags["C_CONTIGUOUS"]
        ctype = dict(QsgParticleSoA._fields_)[name]
        setattr(soa, name, arr.ctypes.data_as(ctype))
    return soa


def soa_from_pointers(ptrs: dict) -> QsgParticleSoA:
    """Build a QsgParticleSoA from raw addresses (e.g. device pointers)."""
    soa = QsgParticleSoA()
    for name in SOA_FIELDS:
        ctype = dict(QsgParticleSoA._fields_)[name]
        setattr(soa, name, C.cast(C.c_void_p(ptrs[name]), ctype))
    return soa


def columns_of(records: np.ndarray) -> dict:
    """Split a PARTICLE_DTYPE record array into contiguous columns."""
    return {name: np.ascontiguousarray(records[name]) for name in SOA_FIELDS}


def records_from_columns(cols: dict, n: int) -> np.ndarray:
    out = np.empty(n, dtype=PARTICLE_DTYPE)
    for name in SOA_FIELDS:
        out[name] = cols[name][:n]
    return out


def empty_columns(n: int) -> dict:
    return {name: np.empty(max(n, 1), dtype=PARTICLE_DTYPE[name]) for name in SOA_FIELDS}
