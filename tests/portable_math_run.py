"""Checks of the portable-math build of the library (libqsg_pm.so) against
the oracle in its portable-math mode and against the reference linked with
the same elementary functions (tests/golden/pm_*.npz).  Run by
tests/test_gpu_portable_math.py in a child process with QSG_LIB=pm (the
library variant is chosen when quicksilver_gb300._native is first imported):

    QSG_LIB=pm python tests/portable_math_run.py functions
    QSG_LIB=pm python tests/portable_math_run.py tracking DECK CYCLES
    QSG_LIB=pm python tests/portable_math_run.py cycles DECK

Each mode asserts and prints one JSON line of what it compared; a failed
check exits non-zero with the assertion's message.
"""
import hashlib
import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent.parent
for p in (ROOT, ROOT / "oracle", ROOT / "tests"):
    sys.path.insert(0, str(p))

import oracle_py as O  # noqa: E402
from helpers import DECKS, assert_flux_close, load_problem, oracle_run, sort_particles  # noqa: E402
from quicksilver_gb300 import _native as N  # noqa: E402
from quicksilver_gb300.monte_carlo import MonteCarlo  # noqa: E402
from quicksilver_gb300.tracker import Tracker  # noqa: E402

GOLDEN = ROOT / "tests" / "golden"
TRACK_SLOTS = [0, 1, 2, 3, 5, 6, 7, 12]


def _sha(recs):
    return hashlib.sha256(np.ascontiguousarray(sort_particles(recs)).tobytes()).hexdigest()


def functions():
    """GPU and CPU evaluate the portable functions to the same bits."""
    rng = np.random.default_rng(5)
    s = rng.integers(0, 2**63, size=1_000_000, dtype=np.uint64) * np.uint64(2) + np.uint64(1)
    r = s.astype(np.float64) * 5.4210108624275222e-20
    x = np.concatenate([r, 2 * 3.14159265 * r, 3.1415926535897932 * (2.0 * r - 1.0),
                        rng.uniform(-1e5, 1e5, 100_000), np.exp(rng.uniform(-700, 700, 100_000)),
                        [0.0, 1.0, 0.5, 5e-324, 1e-310, 3.0, np.pi, -np.pi, 2 * np.pi]])
    got = N.portable_math_eval(x)
    want = O.pm_eval(x)
    for name, g, w in zip(("log", "sin", "cos"), got, want):
        same = (g.view(np.uint64) == w.view(np.uint64)) | (np.isnan(g) & np.isnan(w))
        assert same.all(), f"{name}: {int((~same).sum())} of {len(x)} differ from the CPU"
    return {"arguments": int(len(x)), "bitwise_equal": True}


def tracking(name, cycles):
    """The oracle's particles of each cycle tracked by both: counters, the
    census (every field of every particle) and the flux per (cell, group)."""
    _, sim, hp = load_problem(f"{name}.inp")
    run = oracle_run(hp, sim)
    trk = Tracker(hp)
    worst = 0.0
    try:
        for c in range(cycles):
            run.cycle_init()
            particles = run.processing()
            trk.reset_tallies()
            trk.set_particles(particles)
            trk.track()
            bal, flux = trk.tallies()
            census = trk.census()
            run.cycle_tracking(0)
            np.testing.assert_array_equal(bal[TRACK_SLOTS], run.balance()[TRACK_SLOTS], err_msg=f"cycle {c}")
            assert _sha(census) == _sha(run.processed()), f"cycle {c}: census particles differ"
            worst = max(worst, assert_flux_close(flux, run.flux(), rel=1e-12, scale_floor=0.0))
            assert trk.device_status() == 0
            run.cycle_finalize()
    finally:
        trk.close()
    return {"deck": name, "cycles": cycles, "census_bitwise": True, "flux_worst_over_tolerance": worst}


def cycles(name):
    """Whole device cycles against the reference's own portable-math run:
    the particles after every cycle init and every census bit for bit, all
    13 counters, the flux total."""
    gold = np.load(GOLDEN / f"pm_{name}.npz")
    deck, sim, hp = load_problem(f"{name}.inp")
    mc = MonteCarlo(deck, problem=hp)
    try:
        for c in range(len(gold["balance"])):
            mc.cycle_init()
            assert _sha(mc.processing()) == gold["init_sha"][c], f"cycle {c}: particles after cycle init"
            mc.cycle_tracking()
            assert _sha(mc.tracker.census()) == gold["census_sha"][c], f"cycle {c}: census particles"
            mc.cycle_finalize()
            hist = mc.history(c, 1)
            np.testing.assert_array_equal(hist.balance[0], gold["balance"][c], err_msg=f"cycle {c}")
            assert abs(hist.flux_total[0] - gold["flux_total"][c]) <= 1e-12 * abs(gold["flux_total"][c])
        assert mc.device_status() == 0
    finally:
        mc.close()
    return {"deck": name, "cycles": int(len(gold["balance"])), "particles_bitwise": True}


def main():
    assert N.LIB_PATH.name == "libqsg_pm.so", N.LIB_PATH
    O.use_portable_math(True)
    mode = sys.argv[1]
    if mode == "functions":
        out = functions()
    elif mode == "tracking":
        out = tracking(sys.argv[2], int(sys.argv[3]))
    else:
        out = cycles(sys.argv[2])
    print(json.dumps(out))


if __name__ == "__main__":
    main()
