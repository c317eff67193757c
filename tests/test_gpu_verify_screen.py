"""The FP32 facet screen and the tracking loop's other bit-exact replacements,
checked in the GPU tests by the verification build (libqsg_verify.so,
``python -m quicksilver_gb300.build --verify-screen``; __graft_entry__.build()
makes it beside libqsg.so).

In that build the tracking kernels also evaluate, in the reference's FP64
arithmetic (MCT.cc:280-395, 549-621), every facet the screen skipped and
every facet it accepted without the full test, and compare every integer-pipe
double-to-float conversion and every corrected-reciprocal mean-free-path
quotient with the FP64 operation; any disagreement raises
QSG_DEV_SCREEN_MISS.  Run here on config1 (10 cycles), two cycles of config2,
and the decks whose geometry or boundaries take the screen off the flat,
reflecting case: non-planar hex faces (t_nonflat, whose faces' four facet
planes differ, so the per-face plane bounds carry the proof), reflecting
octant planes (t_scatter_octant), escape boundaries (t_escape, config4),
fission products (t_fission) and the CORAL2-style deck (t_coral1), most at
more particles than the decks hold.  No flag may be raised, and the counters
and flux totals must equal those of the default build (and, at the decks' own
sizes, the unmodified reference's golden counters).
"""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

from helpers import DECKS
from quicksilver_gb300 import _native as N
from quicksilver_gb300.monte_carlo import MonteCarlo

pytestmark = pytest.mark.gpu

ROOT = DECKS.parent.parent
GOLDEN = ROOT / "tests" / "golden"
VERIFY_LIB = N.LIB_PATH.parent / "libqsg_verify.so"


@pytest.fixture(scope="module")
def verify_lib():
    if not VERIFY_LIB.exists():
        from quicksilver_gb300 import build
        build.build(verify_screen=True)
    return VERIFY_LIB


def _verify_run(deck, cycles, particles=None):
    env = dict(os.environ, QSG_LIB="verify")
    extra = [str(particles)] if particles else []
    res = subprocess.run([sys.executable, str(ROOT / "tests" / "verify_screen_run.py"), str(DECKS / deck),
                          str(cycles)] + extra, env=env, capture_output=True, text=True, timeout=900)
    assert res.returncode == 0, res.stderr[-4000:]
    out = json.loads(res.stdout.strip().splitlines()[-1])
    assert out["library"] == "libqsg_verify.so"
    return out


def _default_run(deck, cycles, particles=None):
    from quicksilver_gb300 import Deck
    mc = MonteCarlo(Deck.from_file(DECKS / deck, {"nParticles": particles} if particles else None))
    try:
        hist = mc.run(cycles)
    finally:
        mc.close()
    return hist


@pytest.mark.parametrize("deck,cycles,particles", [
    ("config1.inp", 10, None), ("config2.inp", 2, None),
    ("t_nonflat.inp", 3, None), ("t_nonflat.inp", 3, 200000),
    ("t_scatter_octant.inp", 3, None), ("t_scatter_octant.inp", 3, 200000),
    ("t_escape.inp", 2, None), ("t_fission.inp", 3, None), ("t_fission.inp", 3, 100000),
    ("t_coral1.inp", 5, None), ("config4.inp", 2, 200000)])
def test_verification_build_sees_no_screen_miss(gpu, verify_lib, deck, cycles, particles):
    got = _verify_run(deck, cycles, particles)
    assert got["flags"] & N.QSG_DEV_SCREEN_MISS == 0, "the FP32 screen disagreed with FP64"
    assert got["flags"] == 0, f"device flags 0x{got['flags']:x}"
    want = _default_run(deck, cycles, particles)
    np.testing.assert_array_equal(np.array(got["balance"], dtype=np.uint64), want.balance)
    np.testing.assert_allclose(got["flux_total"], want.flux_total, rtol=1e-12, atol=0)
    assert int(want.balance[:, N.BAL["num_segments"]].sum()) > 0
    golden = GOLDEN / (deck[:-4] + ".npz")
    if particles is None and golden.exists():
        gold = np.load(golden)["balance"][:cycles]   # the fixture may hold more cycles than run here
        assert len(gold) == cycles
        np.testing.assert_array_equal(np.array(got["balance"], dtype=np.uint64), gold)
