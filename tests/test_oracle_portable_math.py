"""The portable elementary functions (quicksilver_gb300/csrc/portable_math.h)
and the oracle's portable-math mode, pinned to the reference linked with the
same functions (make -C oracle ref_pm; fixtures tests/golden/pm_*.npz from
make_golden.py --portable-math).

* The functions are faithful: within one unit in the last place of the host
  libm's log / sin / cos on the random-number stream's arguments (the
  collision azimuth 2 * 3.14159265 * r, CollisionEvent.cc:29; the source
  azimuth pi (2 r - 1), DirectionCosine.cc:9; log r), and equal to it on all
  but a few percent.
* With them the reference's 13 balance counters are the stock reference's on
  every deck (the elementary functions change no event).
* The oracle in portable-math mode is the reference in portable-math mode bit
  for bit: every particle after cycleInit and after cycleTracking (sha256 of
  the sorted sets), every counter, and the flux per (cell, group) within
  1e-12 relative with no floor (only summation order differs).  The GPU
  library built with the same functions is checked against this oracle in
  tests/test_gpu_portable_math.py.
"""
import math

import numpy as np
import pytest

import oracle_py as O
from helpers import DECKS, assert_flux_close, load_problem, oracle_run, sort_particles

GOLDEN = DECKS.parent.parent / "tests" / "golden"
PM_DECKS = ["t_homog", "t_escape", "t_scatter_octant", "t_fission", "t_nonflat", "config1", "config2"]


def _ulps(a, b):
    ia, ib = np.asarray(a).view(np.int64), np.asarray(b).view(np.int64)
    return np.abs(ia - ib)


def _rng_stream(n, seed=1029384756):
    out = np.empty(n)
    s = seed
    for i in range(n):
        s = (2862933555777941757 * s + 3037000493) & 0xFFFFFFFFFFFFFFFF
        out[i] = 5.4210108624275222e-20 * float(s)
    return out


def test_portable_functions_are_faithful():
    r = _rng_stream(200000)
    args = {"log": r, "collision azimuth": 2 * 3.14159265 * r, "source azimuth": 3.1415926535897932 * (2.0 * r - 1.0)}
    lg, _, _ = O.pm_eval(args["log"])
    want = np.array([math.log(v) for v in args["log"]])
    assert _ulps(lg, want).max() <= 1 and (lg != want).mean() < 0.01
    for name in ("collision azimuth", "source azimuth"):
        _, sn, cs = O.pm_eval(args[name])
        ws = np.array([math.sin(v) for v in args[name]])
        wc = np.array([math.cos(v) for v in args[name]])
        assert _ulps(sn, ws).max() <= 1 and (sn != ws).mean() < 0.03, name
        assert _ulps(cs, wc).max() <= 1 and (cs != wc).mean() < 0.03, name
    # special values
    lg, sn, cs = O.pm_eval(np.array([1.0, 0.5, 2.0, 0.0, 5e-324, 0.0, np.pi / 2]))
    assert lg[0] == 0.0 and lg[1] == math.log(0.5) and lg[2] == math.log(2.0)
    assert lg[3] == -np.inf and lg[4] == math.log(5e-324)
    assert sn[5] == 0.0 and cs[5] == 1.0 and sn[6] == 1.0


@pytest.mark.parametrize("name", PM_DECKS[:-1])
def test_portable_math_changes_no_counter_of_the_reference(name):
    pm, stock = np.load(GOLDEN / f"pm_{name}.npz"), np.load(GOLDEN / f"{name}.npz")
    np.testing.assert_array_equal(pm["balance"], stock["balance"])
    np.testing.assert_allclose(pm["flux_total"], stock["flux_total"], rtol=1e-14, atol=0)


@pytest.fixture
def portable_math():
    O.use_portable_math(True)
    try:
        yield
    finally:
        O.use_portable_math(False)


def _sha(recs):
    import hashlib
    return hashlib.sha256(np.ascontiguousarray(sort_particles(recs)).tobytes()).hexdigest()


@pytest.mark.parametrize("name", PM_DECKS)
def test_oracle_portable_math_is_the_reference_bit_for_bit(portable_math, name):
    gold = np.load(GOLDEN / f"pm_{name}.npz")
    _, sim, hp = load_problem(f"{name}.inp", {"nSteps": len(gold["balance"])})
    run = oracle_run(hp, sim)
    for c in range(len(gold["balance"])):
        run.cycle_init()
        assert _sha(run.processing()) == gold["init_sha"][c], f"{name} cycle {c}: particles after cycleInit"
        run.cycle_tracking(0)
        bal = run.balance()
        bal[4] = len(run.processed())   # END, which the reference's dump holds already (cycleFinalize sets it)
        np.testing.assert_array_equal(bal, gold["balance"][c], err_msg=f"{name} cycle {c}")
        assert _sha(run.processed()) == gold["census_sha"][c], f"{name} cycle {c}: census particles"
        flux = run.flux()
        if "flux" in gold and c < len(gold["flux"]):
            assert_flux_close(flux, gold["flux"][c], rel=1e-12, scale_floor=0.0)
        assert_flux_close(flux.sum(axis=1), gold["flux_cell"][c], rel=1e-12)
        assert_flux_close(flux.sum(axis=0), gold["flux_group"][c], rel=1e-12)
        assert abs(flux.sum() - gold["flux_total"][c]) <= 1e-12 * abs(gold["flux_total"][c])
        run.cycle_finalize()
