"""GPU sensitivity tallies (SENS tracking kernel, through the C ABI) against
the oracle's restatement of the same estimator, and the differentiable
binding.

* one tracking call: flux_cell, dflux, leak, dleak vs oracle_track_sens on the
  same particles (counters bit for bit; tallies to summation order: per entry
  1e-12 relative for the forward flux, 1e-10 relative for derivatives, whose
  entries are sums of terms of both signs, each with a floor of 1e-12 x the
  mean entry of that column);
* whole cycles on the device (source, population control, roulette, fission
  passes carry the scores) vs the oracle's cycles;
* the forward run is unchanged by the sensitivity tallies;
* a batch tallies each problem as its single run does;
* torch.autograd: backward = J^T g with J from the same run;
* central finite differences under common random numbers (replicas with
  distinct seeds) agree with the tallied derivatives: every resolved component
  at step 1e-2, the dominant ones at step 1e-4.
"""
import numpy as np
import pytest

import oracle_py as O
from helpers import assert_flux_close, load_problem, oracle_run
from quicksilver_gb300 import Deck
from quicksilver_gb300.monte_carlo import BatchMonteCarlo, MonteCarlo
from quicksilver_gb300.sensitivity import (ABSORPTION, FISSION, SCATTER, Param, band_params, run_sensitivity,
                                           tallies, tie_across_problems)
from quicksilver_gb300.tracker import Tracker

pytestmark = pytest.mark.gpu

DECKS = __import__("pathlib").Path(__file__).resolve().parent.parent / "quicksilver_gb300" / "decks"


def _params(name, hp):
    if name == "t_fission.inp":
        return band_params(hp.array("energies"), hp.num_materials, reactions=(SCATTER, ABSORPTION, FISSION))
    return band_params(hp.array("energies"), hp.num_materials)


def _tuples(params):
    return [(p.material, p.reaction, p.group_lo, p.group_hi, p.theta) for p in params]


def _close_columns(got, want, rel):
    got, want = np.atleast_2d(got), np.atleast_2d(want)
    for k in range(want.shape[1]):
        assert_flux_close(got[:, k], want[:, k], rel=rel, scale_floor=1e-12)


def _compare(gpu, want_fc, want_df, want_leak, want_dl):
    assert_flux_close(gpu["flux_cell"], want_fc, rel=1e-12, scale_floor=1e-12)
    _close_columns(gpu["dflux"], want_df, rel=1e-10)
    np.testing.assert_allclose(gpu["leak"][0], want_leak, rtol=1e-12, atol=0)
    np.testing.assert_allclose(gpu["dleak"][0], want_dl, rtol=1e-10, atol=1e-12 * max(abs(want_leak), 1.0))


@pytest.mark.parametrize("name", ["t_sens.inp", "t_fission.inp", "t_nonflat.inp"])
def test_gpu_sens_tracking_matches_oracle(gpu, name):
    _, sim, hp = load_problem(name)
    params = _params(name, hp)
    run = oracle_run(hp, sim)
    run.cycle_init()
    parts = run.processing()
    want = O.track_sens(hp.ptr, hp.num_cells, hp.num_groups, parts, _tuples(params))
    trk = Tracker(hp)
    try:
        trk.enable_sensitivity(params)
        trk.set_particles(parts)
        trk.track()
        bal, flux = trk.tallies()
        np.testing.assert_array_equal(bal, want["balance"])
        got = trk.read_sensitivity()
        _compare(got, want["flux_cell"], want["dflux"], want["leak"], want["dleak"])
        assert np.abs(want["dflux"]).sum() > 0
        assert trk.device_status() == 0
    finally:
        trk.close()


@pytest.mark.parametrize("name", ["t_sens.inp", "t_fission.inp"])
def test_gpu_sens_cycles_match_oracle(gpu, name):
    deck, sim, hp = load_problem(name)
    params = _params(name, hp)
    run = oracle_run(hp, sim)
    run.enable_sensitivity(_tuples(params))
    for _ in range(sim.n_steps):
        run.cycle_init()
        run.cycle_tracking(0)
        run.cycle_finalize()
    fc, df, leak, dl = run.read_sensitivity()
    mc = MonteCarlo(deck, problem=hp)
    try:
        mc.tracker.enable_sensitivity(params)
        mc.run()
        got = mc.tracker.read_sensitivity()
    finally:
        mc.close()
    _compare(got, fc, df, leak, dl)


def test_gpu_forward_unchanged_by_sensitivities(gpu):
    deck = Deck.from_file(DECKS / "t_sens.inp")
    hp = deck.build()
    a = MonteCarlo(deck, problem=hp)
    b = MonteCarlo(deck, problem=hp)
    try:
        b.tracker.enable_sensitivity(band_params(hp.array("energies"), hp.num_materials))
        ha, hb = a.run(), b.run()
        np.testing.assert_array_equal(ha.balance, hb.balance)
        np.testing.assert_allclose(hb.flux_total, ha.flux_total, rtol=1e-12, atol=0)
        # the per-cell forward tally is the group sum of the per-cycle flux
        assert abs(b.tracker.read_sensitivity()["flux_cell"].sum() - hb.flux_total.sum()) <= \
            1e-12 * hb.flux_total.sum()
    finally:
        a.close()
        b.close()


def test_gpu_sens_batch_matches_single(gpu):
    deck = Deck.from_file(DECKS / "t_sens.inp")
    offsets = [0, 12345]
    probs = [deck.build(), deck.build()]
    base = band_params(probs[0].array("energies"), probs[0].num_materials)
    bmc = BatchMonteCarlo([deck, deck], problems=probs, seed_offsets=offsets)
    try:
        params = tie_across_problems(base, bmc.tracker.material_offsets())
        bmc.tracker.enable_sensitivity(params)
        bmc.run(deck.simulation.n_steps, use_graph=True)
        got = bmc.tracker.read_sensitivity()
        coff = bmc.tracker.cell_offsets
    finally:
        bmc.close()
    for q in range(2):
        single = run_sensitivity(deck, base, seed_offset=offsets[q])
        cells = slice(int(coff[q]), int(coff[q + 1]))
        assert_flux_close(got["flux_cell"][cells], single["flux_cell"], rel=1e-12, scale_floor=1e-12)
        _close_columns(got["dflux"][cells], single["dflux"], rel=1e-10)
        np.testing.assert_allclose(got["leak"][q], single["leak"][0], rtol=1e-12)
        np.testing.assert_allclose(got["dleak"][q], single["dleak"][0], rtol=1e-10, atol=1e-12 * single["leak"][0])


def test_gpu_autograd_backward(gpu):
    torch = pytest.importorskip("torch")
    deck = Deck.from_file(DECKS / "t_sens.inp")
    hp = deck.build()
    params = band_params(hp.array("energies"), hp.num_materials)
    K = len(params)
    theta = torch.linspace(0.9, 1.1, K, dtype=torch.float64).requires_grad_(True)
    flux, leak = tallies(theta, deck, params)
    w = torch.linspace(0.0, 1.0, flux.numel(), dtype=torch.float64)
    loss = (w * flux).sum() + 3.0 * leak.sum()
    loss.backward()
    from quicksilver_gb300.sensitivity import with_theta
    ref = run_sensitivity(deck, with_theta(params, theta.detach().numpy()))
    want = ref["dflux"].T @ w.numpy() + 3.0 * ref["dleak"][0]
    np.testing.assert_allclose(theta.grad.numpy(), want, rtol=1e-9, atol=1e-12 * np.abs(want).max())
    np.testing.assert_allclose(flux.detach().numpy(), ref["flux_cell"], rtol=1e-12, atol=0)


def _crn_differences(h, R, n_particles=100000):
    """Per replica (distinct seed offsets): tallied derivatives and central
    differences (step h, common random numbers) of total flux and leakage."""
    deck = Deck.from_file(DECKS / "t_sens.inp", {"nParticles": str(n_particles)})
    hp = deck.build()
    params = band_params(hp.array("energies"), hp.num_materials)
    K = len(params)
    lr = np.zeros((R, 2, K))
    fd = np.zeros((R, 2, K))
    base = np.zeros((R, 2))
    for i in range(R):
        off = 7919 * (i + 1)
        res = run_sensitivity(deck, params, seed_offset=off)
        lr[i, 0] = res["dflux"].sum(axis=0)
        lr[i, 1] = res["dleak"][0]
        base[i] = (res["flux_cell"].sum(), res["leak"][0])
        for k in range(K):
            vals = []
            for sgn in (1.0, -1.0):
                shifted = [p if j != k else Param(p.material, p.reaction, p.group_lo, p.group_hi, 1.0 + sgn * h)
                           for j, p in enumerate(params)]
                out = run_sensitivity(deck, shifted, seed_offset=off)
                vals.append((out["flux_cell"].sum(), out["leak"][0]))
            fd[i, 0, k] = (vals[0][0] - vals[1][0]) / (2 * h)
            fd[i, 1, k] = (vals[0][1] - vals[1][1]) / (2 * h)
    # summation-order rounding of the tallies (~1e-13 relative) is not an event flip
    flips = (np.abs(fd) > 1e-9 * np.abs(base)[:, :, None] / (2 * h)).sum(axis=0)
    d = lr - fd
    se_d = d.std(axis=0, ddof=1) / np.sqrt(R)
    z = np.abs(d.mean(axis=0)) / np.where(se_d > 0, se_d, np.inf)
    return lr, fd, flips, z


def _report(z, compared, lr, fd):
    R = lr.shape[0]
    return (f"z {z}\ncompared {compared}\nscores {lr.mean(axis=0)}\nfd {fd.mean(axis=0)}\n"
            f"fd se {fd.std(axis=0, ddof=1) / np.sqrt(R)}")


def test_gpu_sens_vs_crn_finite_differences_step_1e2(gpu):
    """Step 1e-2: every component whose central differences saw event flips in
    at least 3/4 of 48 replicas agrees with the tallied derivative within 4.5
    standard errors (the O(h^2) bias is ~1e-4 relative, far below them)."""
    lr, fd, flips, z = _crn_differences(1e-2, 48)
    compared = flips >= 36
    assert compared.sum() >= 16, flips
    assert (z[compared] <= 4.5).all(), _report(z, compared, lr, fd)


def test_gpu_sens_vs_crn_finite_differences_step_1e4(gpu):
    """Step 1e-4: a difference is nonzero only when an event flips between the
    two runs, so its replica distribution is a spike at zero plus rare large
    values, and its sample mean converges only where flips are frequent.
    Compared: components whose differences are resolved at this sample size
    (flips in every replica, replica mean beyond 5 of its standard errors) --
    the dominant sensitivities; all of them agree within 4.5 standard errors."""
    lr, fd, flips, z = _crn_differences(1e-4, 24)
    R = lr.shape[0]
    se_fd = fd.std(axis=0, ddof=1) / np.sqrt(R)
    compared = (flips == R) & (np.abs(fd.mean(axis=0)) > 5 * se_fd)
    assert compared.sum() >= 3, _report(z, compared, lr, fd)
    assert (z[compared] <= 4.5).all(), _report(z, compared, lr, fd)
