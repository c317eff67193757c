"""qsg_track_host: particles tracked straight from, and census particles
written straight to, page-locked host arrays (no staging copies; the GPU
reads and writes them over the host link while it tracks).  The results must
be those of the staged calls (qsg_set_particles + qsg_track_cycle +
qsg_get_census) on the same particles: counters bit for bit, census particles
byte for byte (their order aside), flux to summation order, the input arrays
untouched.  Error paths: pageable arrays, a census that does not fit,
sensitivities switched on."""
import numpy as np
import pytest

from helpers import assert_flux_close, load_problem, oracle_run
from quicksilver_gb300 import _native as N
from quicksilver_gb300.sensitivity import band_params
from quicksilver_gb300.tracker import Tracker

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

_TORCH = {"<f8": torch.float64, "<u8": torch.int64, "<i4": torch.int32}


def _pinned(n, records=None):
    """Page-locked SoA columns with room for n particles (filled from records)."""
    cols = {name: torch.zeros(max(n, 1), dtype=_TORCH[N.PARTICLE_DTYPE[name].str], pin_memory=True)
            for name in N.SOA_FIELDS}
    if records is not None:
        for name, t in cols.items():
            t.numpy().view(N.PARTICLE_DTYPE[name])[:len(records)] = records[name]
    return cols


def _records(cols, n):
    return N.records_from_columns({k: t.numpy().view(N.PARTICLE_DTYPE[k]) for k, t in cols.items()}, n)


def _sorted(recs):
    return recs[np.lexsort((recs["random_number_seed"], recs["identifier"]))]


def _source(name):
    deck, sim, hp = load_problem(name)
    run = oracle_run(hp, sim)
    run.cycle_init()
    parts = np.ascontiguousarray(run.processing(), dtype=N.PARTICLE_DTYPE)
    return hp, parts


@pytest.mark.parametrize("name", ["t_fission.inp", "t_homog.inp", "t_nonflat.inp"])
def test_track_host_matches_staged_calls(gpu, name):
    hp, parts = _source(name)
    n = len(parts)
    staged, direct = Tracker(hp), Tracker(hp)
    try:
        staged.set_particles(parts)
        staged.track()
        want_census = staged.census()
        want_bal, want_flux = staged.tallies()
        cap = 2 * len(want_census) + 1024   # fission multiplies the population
        inp, out = _pinned(n, parts), _pinned(cap)
        got_n = direct.track_host(inp, n, out, cap)
        bal, flux = direct.tallies()
        np.testing.assert_array_equal(bal, want_bal)
        assert_flux_close(flux, want_flux, rel=1e-12)
        assert got_n == len(want_census)
        assert _sorted(_records(out, got_n)).tobytes() == _sorted(want_census).tobytes()
        assert _records(inp, n).tobytes() == parts.tobytes()
        assert direct.device_status() == 0
        if name == "t_fission.inp":
            assert bal[N.BAL["produce"]] > 0   # more than one pass
    finally:
        staged.close()
        direct.close()


def test_track_host_errors(gpu):
    hp, parts = _source("t_fission.inp")   # ~7e4 census particles
    n = len(parts)
    trk = Tracker(hp)
    try:
        with pytest.raises(N.QsgError) as ei:   # pageable numpy arrays
            trk.track_host(N.columns_of(parts), n, N.empty_columns(4 * n), 4 * n)
        assert ei.value.code == N.QSG_ERR_INVALID and "pageable" in str(ei.value)
        inp, small = _pinned(n, parts), _pinned(64)
        with pytest.raises(N.QsgError) as ei:
            trk.track_host(inp, n, small, 64)
        assert ei.value.code == N.QSG_ERR_CAPACITY and "census_capacity" in str(ei.value)
        assert trk.device_status() & N.QSG_DEV_STORE_OVERFLOW
        assert trk.track_host(inp, 0, small, 64) == 0
        with pytest.raises(N.QsgError) as ei:   # census written over the particles still being read
            trk.track_host(inp, n, inp, n)
        assert ei.value.code == N.QSG_ERR_INVALID and "overlap" in str(ei.value)
        trk.enable_sensitivity(band_params(hp.array("energies"), hp.num_materials))
        with pytest.raises(N.QsgError) as ei:
            trk.track_host(inp, n, _pinned(4 * n), 4 * n)
        assert ei.value.code == N.QSG_ERR_UNSUPPORTED
    finally:
        trk.close()
