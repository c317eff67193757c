"""qsg_track_particles_noalloc (tracking with no device allocation) through
the C ABI: against qsg_track_cycle_sync and directly against the C oracle,
with either tracking kernel, on two calls in a row; and its refusals --
census overflow, too many fission products, host pointers, overlapping
arrays -- each followed by a call that is exact again.

The file name makes pytest collect it last, so in a full run it follows every
other GPU test in the same process; run alone, its first call is also the
first in the process's CUDA context (the call that looks up the scratch
array's address).  Inputs and outputs are device arrays that the test (the
caller) allocates with torch; the entry point itself allocates nothing, which
the test checks through the device's free memory across every call.
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
        free_before = torch.cuda.mem_get_info()[0]
        code = N.lib().qsg_track_particles_noalloc(
            self.trk.handle, C.byref(_soa(self.inputs)), self.n, C.byref(_soa(self.census)), self.cap,
            C.byref(n_census), self.flux.data_ptr(), self.balance.data_ptr(), stream)
        torch.cuda.synchronize()
        free_after = torch.cuda.mem_get_info()[0]
        assert free_after >= free_before - (1 << 20), "device memory was taken during the call"
        N.check(code)
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


@pytest.mark.parametrize("deck,kernel", [("t_fission.inp", 1), ("t_nonflat.inp", 1), ("t_fission.inp", 0)])
def test_noalloc_matches_track_cycle_sync(gpu, deck, kernel):
    """Against the existing entry point with the same kernel selected (1: the
    warp-pool kernel, the default; 0: one history per lane), twice in a row:
    the second call finds the first call's contents in the scratch and must
    clear them itself."""
    torch = _torch()
    hp, particles = _source_particles(deck)
    trk = Tracker(hp)
    try:
        trk.set_track_kernel(kernel)
        want = _existing(trk, particles)
        call = NoAllocCall(torch, trk, particles, census_capacity=4 * len(want[2]) + 1024)
        _compare(call(), want)
        _compare(call(), want)
        assert trk.device_status() == 0
    finally:
        trk.close()


def test_noalloc_matches_oracle_on_fission(gpu):
    """Directly against the oracle on the fission deck (products re-tracked
    in later passes through the scratch): all tracking counters -- fission
    and produce included -- bit for bit."""
    torch = _torch()
    _, sim, hp = load_problem("t_fission.inp")
    run = oracle_run(hp, sim)
    run.cycle_init()
    particles = run.processing()
    run.cycle_tracking(0)
    want = (run.balance(), run.flux(), run.processed())
    trk = Tracker(hp)
    try:
        # fission grows the population over the passes: room for all of it
        call = NoAllocCall(torch, trk, particles, census_capacity=len(want[2]) + 1024)
        bal, flux, census = call()
        slots = [0, 1, 2, 3, 5, 6, 7, 12]
        np.testing.assert_array_equal(bal[slots], want[0][slots])
        assert int(bal[5]) > 0 and int(bal[6]) > 0            # fission happened, products were tracked
        _compare((bal, flux, census), (bal, want[1], want[2]))
    finally:
        trk.close()


def test_noalloc_refusals_leave_next_call_exact(gpu):
    """Census beyond census_capacity: QSG_ERR_CAPACITY (the census arrays
    hold their first census_capacity particles); a host (numpy) array or
    arrays that overlap: QSG_ERR_INVALID before any work; n = 0: nothing to
    do.  The next full call is exact each time."""
    torch = _torch()
    hp, particles = _source_particles("t_nonflat.inp")
    trk = Tracker(hp)
    try:
        want = _existing(trk, particles)
        good = NoAllocCall(torch, trk, particles, census_capacity=4 * len(want[2]) + 1024)
        small = NoAllocCall(torch, trk, particles, census_capacity=len(want[2]) // 2)
        with pytest.raises(N.QsgError) as exc:
            small()
        assert exc.value.code == N.QSG_ERR_CAPACITY and "census_capacity" in str(exc.value)
        _compare(good(), want)

        n_census = C.c_uint64(7)
        host_x = np.zeros(len(particles))
        bad = dict(good.inputs)
        bad["x"] = host_x
        soa_bad = N.soa_from_pointers({k: (v.ctypes.data if isinstance(v, np.ndarray) else v.data_ptr())
                                       for k, v in bad.items()})
        code = N.lib().qsg_track_particles_noalloc(trk.handle, C.byref(soa_bad), good.n, C.byref(_soa(good.census)),
                                                   good.cap, C.byref(n_census), good.flux.data_ptr(),
                                                   good.balance.data_ptr(), None)
        assert code == N.QSG_ERR_INVALID and n_census.value == 0
        _compare(good(), want)

        # the census written over the particles (an in-place call)
        code = N.lib().qsg_track_particles_noalloc(trk.handle, C.byref(_soa(good.inputs)), good.n,
                                                   C.byref(_soa(good.inputs)), good.n, C.byref(n_census),
                                                   good.flux.data_ptr(), good.balance.data_ptr(), None)
        assert code == N.QSG_ERR_INVALID
        # flux on top of the balance counters
        code = N.lib().qsg_track_particles_noalloc(trk.handle, C.byref(_soa(good.inputs)), good.n,
                                                   C.byref(_soa(good.census)), good.cap, C.byref(n_census),
                                                   good.flux.data_ptr(), good.flux.data_ptr(), None)
        assert code == N.QSG_ERR_INVALID
        _compare(good(), want)

        n_census = C.c_uint64(7)
        N.check(N.lib().qsg_track_particles_noalloc(trk.handle, C.byref(_soa(good.inputs)), 0,
                                                    C.byref(_soa(good.census)), good.cap, C.byref(n_census),
                                                    good.flux.data_ptr(), good.balance.data_ptr(), None))
        assert n_census.value == 0
        _compare(good(), want)
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
