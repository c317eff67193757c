"""qsg_track_particles_noalloc (tracking with no device allocation) against
qsg_track_cycle_sync, both through the C ABI.

The file name makes pytest collect it last, so in a full run it follows every
other GPU test in the same process; run alone, its first call is also the
first on the device (the call that looks up the scratch array's address).
Inputs and outputs are device arrays that the test (the caller) allocates
with torch; the entry point itself allocates nothing.
"""
import ctypes as C

import numpy as np
import pytest

from helpers import assert_flux_close, load_problem, oracle_run, sort_particles
from quicksilver_gb300 import _native as N
from quicksilver_gb300.tracker import Tracker

pytestmark = pytest.mark.gpu

FP_FIELDS = ["x", "y", "z", "vx", "vy", "vz", "kinetic_energy", "weight", "time_to_census", "age",
             "num_mean_free_paths", "num_segments"]
INT_FIELDS = ["random_number_seed", "identifier", "last_event", "num_collisions", "breed", "species",
              "domain", "cell"]


def _torch():
    return pytest.importorskip("torch")


def _as_device(torch, arr):
    arr = np.ascontiguousarray(arr)
    if arr.dtype == np.uint64:
        arr = arr.view(np.int64)
    return torch.from_numpy(arr).cuda()


def _soa(tensors):
    return N.soa_from_pointers({k: t.data_ptr() for k, t in tensors.items()})


def _empty_store(torch, cap):
    out = {}
    for name in N.SOA_FIELDS:
        dt = N.PARTICLE_DTYPE[name]
        tdt = torch.float64 if dt.kind == "f" else (torch.int64 if dt.itemsize == 8 else torch.int32)
        out[name] = torch.empty(cap, dtype=tdt, device="cuda")
    return out


def _records(tensors, n):
    recs = np.empty(n, dtype=N.PARTICLE_DTYPE)
    for name in N.SOA_FIELDS:
        col = tensors[name][:n].cpu().numpy()
        recs[name] = col.view(np.uint64) if N.PARTICLE_DTYPE[name] == np.uint64 else col
    return recs


class NoAllocCall:
    """Device inputs of one particle set and preallocated outputs, reused by every call."""

    def __init__(self, torch, trk, particles, census_capacity):
        self.torch, self.trk = torch, trk
        self.n = len(particles)
        self.inputs = {k: _as_device(torch, v) for k, v in N.columns_of(particles).items()}
        self.census = _empty_store(torch, census_capacity)
        self.cap = census_capacity
        self.flux = torch.zeros(trk.num_cells * trk.num_groups, dtype=torch.float64, device="cuda")
        self.balance = torch.zeros(len(trk.problems) * 13, dtype=torch.int64, device="cuda")

    def __call__(self):
        torch = self.torch
        self.flux.zero_()
        self.balance.zero_()
        stream = torch.cuda.current_stream().cuda_stream
        torch.cuda.synchronize()
        n_census = C.c_uint64(0)
        N.check(N.lib().qsg_track_particles_noalloc(
            self.trk.handle, C.byref(_soa(self.inputs)), self.n, C.byref(_soa(self.census)), self.cap,
            C.byref(n_census), self.flux.data_ptr(), self.balance.data_ptr(), stream))
        torch.cuda.synchronize()
        bal = self.balance.cpu().numpy().view(np.uint64).reshape(-1, 13).sum(axis=0, dtype=np.uint64)
        flux = self.flux.cpu().numpy().reshape(self.trk.num_cells, self.trk.num_groups)
        return bal, flux, _records(self.census, n_census.value)


def _existing(trk, particles):
    trk.reset_tallies()
    trk.set_particles(particles)
    trk.track()
    bal, flux = trk.tallies()
    return bal, flux, trk.census()


def _compare(got, want):
    bal, flux, census = got
    want_bal, want_flux, want_census = want
    np.testing.assert_array_equal(bal, want_bal)
    # the GPU tests' flux tolerance: 1e-12 relative per (cell, group), with a
    # floor of 1e-12 x the mean entry; marginals and total 1e-12 relative
    assert_flux_close(flux, want_flux, rel=1e-12, scale_floor=1e-12)
    assert_flux_close(flux.sum(axis=1), want_flux.sum(axis=1), rel=1e-12)
    assert abs(flux.sum() - want_flux.sum()) <= 1e-12 * abs(want_flux.sum())
    assert len(census) == len(want_census)
    g, w = sort_particles(census), sort_particles(want_census)
    for f in INT_FIELDS:
        np.testing.assert_array_equal(g[f], w[f], err_msg=f)
    for f in FP_FIELDS:
        np.testing.assert_allclose(g[f], w[f], rtol=1e-7, atol=1e-12, err_msg=f)


def _source_particles(deck, overrides=None):
    _, sim, hp = load_problem(deck, overrides)
    run = oracle_run(hp, sim)
    run.cycle_init()
    return hp, run.processing()


@pytest.mark.parametrize("deck", ["t_fission.inp", "t_nonflat.inp"])
def test_noalloc_matches_track_cycle_sync(gpu, deck):
    torch = _torch()
    hp, particles = _source_particles(deck)
    trk = Tracker(hp)
    try:
        want = _existing(trk, particles)
        call = NoAllocCall(torch, trk, particles, census_capacity=4 * len(want[2]) + 1024)
        _compare(call(), want)
        # second call in a row: the scratch still holds the first call's
        # contents and must be cleared by the call itself
        free_before = torch.cuda.mem_get_info()[0]
        second = call()
        free_after = torch.cuda.mem_get_info()[0]
        _compare(second, want)
        assert free_after >= free_before - (1 << 20), "device memory was taken during the call"
        assert trk.device_status() == 0
    finally:
        trk.close()


def test_noalloc_rejects_too_many_products(gpu):
    """A pass with more fission products than QSG_NOALLOC_MAX_PRODUCTS ends
    the call with QSG_ERR_CAPACITY; the next call still gives exact results."""
    torch = _torch()
    hp, big = _source_particles("t_fission.inp", {"nParticles": "100000"})
    trk = Tracker(hp)
    try:
        call = NoAllocCall(torch, trk, big, census_capacity=8 * len(big))
        with pytest.raises(N.QsgError) as exc:
            call()
        assert exc.value.code == N.QSG_ERR_CAPACITY
        assert "QSG_NOALLOC_MAX_PRODUCTS" in str(exc.value)
        _, small = _source_particles("t_fission.inp")
        want = _existing(trk, small)
        call = NoAllocCall(torch, trk, small, census_capacity=4 * len(want[2]) + 1024)
        _compare(call(), want)
    finally:
        trk.close()
