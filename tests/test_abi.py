"""CPU-side checks of the C ABI: the library loads without a GPU, exports
every function include/qsg.h declares, and its host-only entry points (deck
reader, table builder, error reporting) behave like the reference's."""
import ctypes
import re

import numpy as np
import pytest

from helpers import DECKS
from quicksilver_gb300 import Deck
from quicksilver_gb300 import _native as N

HEADER = DECKS.parent.parent / "include" / "qsg.h"


def declared_functions():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"^int\s+(qsg_\w+)\s*\(", text, flags=re.M)))


def test_library_exports_every_declared_symbol(native_lib):
    names = declared_functions()
    assert len(names) >= 30
    for name in names:
        assert hasattr(native_lib, name), f"{name} declared in qsg.h but not exported"


def test_nvtx_build_exports_the_same_abi():
    """The variant with NVTX ranges around its phases (build.py --nvtx,
    -DQSG_NVTX, as the reference's -DUSE_NVTX) builds and exports the same
    functions."""
    from quicksilver_gb300 import build
    lib = ctypes.CDLL(str(build.build(nvtx=True)))
    for name in declared_functions():
        assert hasattr(lib, name), name
    assert lib.qsg_abi_version() == 1


def test_abi_version(native_lib):
    assert native_lib.qsg_abi_version() == 1


def test_bad_deck_reports_error():
    with pytest.raises(N.QsgError) as ei:
        Deck.from_string("Geometry:\n   material: x\n   shape: cone\n")
    assert ei.value.code == N.QSG_ERR_INVALID and "brick or sphere" in str(ei.value)
    with pytest.raises(N.QsgError) as ei:
        Deck.from_file("/nonexistent/deck.inp")
    assert ei.value.code == N.QSG_ERR_IO


def test_default_problem_and_overrides():
    # no Geometry block: supplyDefaults (Parameters.cc:350-379)
    d = Deck.from_string("Simulation:\n   nx: 2\n   ny: 2\n   nz: 2\n   nGroups: 4\n", {"lx": 4, "ly": 4, "lz": 4})
    s = d.simulation
    assert (s.nx, s.n_groups, s.lx) == (2, 4, 4.0)
    hp = d.build()
    assert hp.num_materials == 1 and hp.num_cells == 8
    assert np.all(hp.array("cell_volume") > 0)
    with pytest.raises(N.QsgError):
        d.set("noSuchKey", 1)


def test_create_without_gpu_fails_loudly(has_gpu):
    if has_gpu:
        pytest.skip("a GPU is visible")
    _, _, hp = None, None, Deck.from_file(DECKS / "t_homog.inp").build()
    h = ctypes.c_void_p()
    rc = N.lib().qsg_create(ctypes.byref(hp.view), None, ctypes.byref(h))
    assert rc == N.QSG_ERR_NO_DEVICE and "no CUDA device" in N.last_error()


def test_new_entry_points_check_arguments_before_any_cuda_call(native_lib):
    """Null handles and arguments are reported, not dereferenced (no GPU needed)."""
    lib = N.lib()
    got = ctypes.c_uint64(7)
    assert lib.qsg_track_host(None, None, 0, None, 0, ctypes.byref(got), None) == N.QSG_ERR_INVALID
    assert lib.qsg_set_exponential_tally(None, 1) == N.QSG_ERR_INVALID
    assert lib.qsg_read_cell_tally(None, None) == N.QSG_ERR_INVALID
    assert "null" in N.last_error()
    assert lib.qsg_check_arithmetic(0, 16, 1, None) == N.QSG_ERR_INVALID
    out = (ctypes.c_uint64 * 4)()
    assert lib.qsg_check_arithmetic(-1, 16, 1, out) in (N.QSG_ERR_INVALID, N.QSG_ERR_NO_DEVICE)
    assert lib.qsg_portable_math_eval(0, None, 4, None, None, None) == N.QSG_ERR_INVALID


@pytest.mark.parametrize("name", ["t_homog.inp", "t_scatter_octant.inp", "t_nonflat.inp", "config1.inp"])
def test_problem_check_accepts_built_decks(name):
    hp = Deck.from_file(DECKS / name).build()
    assert N.lib().qsg_problem_check(ctypes.byref(hp.view)) == N.QSG_OK, N.last_error()


def test_problem_check_runs_the_reference_mesh_self_test():
    """consistencyCheck (initMC.cc:202-234): a facet whose neighbour does not
    lead back to it is rejected before any device is touched."""
    hp = Deck.from_file(DECKS / "t_homog.inp").build()
    view = N.QsgProblem.from_buffer_copy(hp.view)
    adj = hp.array("facet_adjacent_facet").astype(np.int32).copy()
    cells = hp.array("facet_adjacent_cell")
    inner = int(np.nonzero(cells != np.repeat(np.arange(hp.num_cells), 24))[0][0])   # an interior facet
    adj[inner] = (adj[inner] + 1) % 24
    view.facet_adjacent_facet = adj.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
    assert N.lib().qsg_problem_check(ctypes.byref(view)) == N.QSG_ERR_INVALID
    assert "not symmetric" in N.last_error()
    assert N.lib().qsg_problem_check(None) == N.QSG_ERR_INVALID
