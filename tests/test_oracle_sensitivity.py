"""The oracle's sensitivity scores (CPU restatement of the SENS tracking
kernel's differential-operator tallies) on their own: forward tracking is
unchanged by them, parameters that scale nothing get zero derivatives, a
rescaled parameterisation rescales the derivatives exactly, and the
derivatives agree with common-random-number central finite differences of the
same tallies (replica statistics)."""
import numpy as np

import oracle_py as O
from helpers import load_problem, oracle_run
from quicksilver_gb300.sensitivity import band_params

DECK = "t_sens.inp"


def _params(hp, theta=1.0):
    return [(p.material, p.reaction, p.group_lo, p.group_hi, theta)
            for p in band_params(hp.array("energies"), hp.num_materials)]


def _source(hp, sim, cycles=1):
    """Processing particles of successive cycle inits (fresh source streams each)."""
    run = oracle_run(hp, sim)
    out = []
    for _ in range(cycles):
        run.cycle_init()
        out.append(run.processing())
    return out


def test_forward_unchanged_by_scores():
    _, sim, hp = load_problem(DECK)
    parts = _source(hp, sim)[0]
    census, bal, flux = O.track(hp.ptr, hp.num_cells, hp.num_groups, parts)
    res = O.track_sens(hp.ptr, hp.num_cells, hp.num_groups, parts, _params(hp))
    np.testing.assert_array_equal(res["balance"], bal)
    key = lambda r: np.lexsort((r["random_number_seed"], r["identifier"]))
    a, b = census[key(census)], res["census"][key(res["census"])]
    assert a.tobytes() == b.tobytes()
    # the group-summed flux is the same track-length tally
    np.testing.assert_allclose(res["flux_cell"], flux.sum(axis=1), rtol=1e-12, atol=0)
    np.testing.assert_allclose(res["flux"], flux, rtol=1e-12, atol=0)
    assert res["leak"] > 0 and bal[2] > 0


def test_parameter_scaling_nothing_has_zero_derivative():
    _, sim, hp = load_problem(DECK)
    parts = _source(hp, sim)[0]
    params = _params(hp) + [(0, 3, 0, hp.num_groups, 1.0)]   # no fission reactions in this deck
    res = O.track_sens(hp.ptr, hp.num_cells, hp.num_groups, parts, params)
    assert not res["dflux"][:, -1].any() and res["dleak"][-1] == 0.0
    assert not res["census_scores"][:, -1].any()
    assert np.abs(res["dflux"][:, :-1]).sum() > 0


def test_rescaled_parameterisation():
    """Tables scaled by c at theta = c, or baked in at theta = 1: identical
    histories, derivatives differ by exactly the factor c (up to rounding)."""
    _, sim, hp = load_problem(DECK)
    parts = _source(hp, sim)[0]
    c = 1.25
    base = _params(hp)
    k = 3   # material 0, absorption, high band
    m, r, lo, hi, _ = base[k]
    _, _, hp_c = load_problem(DECK)
    hp_c.scale_xs(m, r, lo, hi, c)
    at_c = [p if j != k else (m, r, lo, hi, c) for j, p in enumerate(base)]
    a = O.track_sens(hp_c.ptr, hp.num_cells, hp.num_groups, parts, at_c)
    b = O.track_sens(hp_c.ptr, hp.num_cells, hp.num_groups, parts, base)
    np.testing.assert_array_equal(a["balance"], b["balance"])
    np.testing.assert_allclose(b["dflux"][:, k], c * a["dflux"][:, k], rtol=1e-9,
                               atol=1e-12 * np.abs(b["dflux"][:, k]).max())
    np.testing.assert_allclose(b["dleak"][k], c * a["dleak"][k], rtol=1e-9)
    others = [j for j in range(len(base)) if j != k]
    # other parameters: the same sums, up to OpenMP summation order
    np.testing.assert_allclose(b["dflux"][:, others], a["dflux"][:, others], rtol=1e-12,
                               atol=1e-12 * np.abs(a["dflux"][:, others]).max())


def test_scores_match_crn_finite_differences():
    """d(total flux)/dtheta and d(leakage)/dtheta: per replica, the score
    estimate and the CRN central difference (step 1e-2) estimate the same
    derivative; their mean difference over 40 replicas must be within 4.5
    standard errors for every parameter."""
    deck, sim, hp = load_problem(DECK)
    params = _params(hp)
    K = len(params)
    h = 1e-2
    shifted = []
    for (m, r, lo, hi, _) in params:
        pair = []
        for sgn in (1.0, -1.0):
            _, _, hq = load_problem(DECK)
            hq.scale_xs(m, r, lo, hi, 1.0 + sgn * h)
            pair.append(hq)
        shifted.append(pair)
    R = 40
    lr = np.zeros((R, 2, K))
    fd = np.zeros((R, 2, K))
    for i, parts in enumerate(_source(hp, sim, R)):
        res = O.track_sens(hp.ptr, hp.num_cells, hp.num_groups, parts, params)
        lr[i, 0] = res["dflux"].sum(axis=0)
        lr[i, 1] = res["dleak"]
        for k in range(K):
            vals = []
            for hq in shifted[k]:
                out = O.track_sens(hq.ptr, hq.num_cells, hq.num_groups, parts, params)
                vals.append((out["flux_cell"].sum(), out["leak"]))
            fd[i, 0, k] = (vals[0][0] - vals[1][0]) / (2 * h)
            fd[i, 1, k] = (vals[0][1] - vals[1][1]) / (2 * h)
    d = lr - fd
    se = d.std(axis=0, ddof=1) / np.sqrt(R)
    mean = d.mean(axis=0)
    # a central difference that never saw an event flip in any replica (all
    # zero, e.g. the leakage of an inner region's absorption) carries no
    # information; every other component is compared
    informative = fd.std(axis=0, ddof=1) > 0
    assert informative[0].all() and informative.sum() >= 18
    ok = (np.abs(mean) <= 4.5 * se) | ~informative
    assert ok.all(), f"score vs finite-difference mismatch:\nmean diff {mean}\nse {se}\nscore mean {lr.mean(axis=0)}"
    # the estimator is not trivially zero where the tallies depend on theta
    assert (np.abs(lr.mean(axis=0)[0]) > 3 * lr.std(axis=0, ddof=1)[0] / np.sqrt(R)).sum() >= 4
