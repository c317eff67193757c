"""The GPU library built with the portable elementary functions
(libqsg_pm.so: ``python -m quicksilver_gb300.build --portable-math``;
__graft_entry__.build() makes it beside libqsg.so) tracks exactly the
reference's trajectories when the reference uses the same functions.

The default build takes log / sin / cos from the CUDA math library, which
rounds a few arguments per thousand differently from the host libm the
reference uses: counters stay bit for bit, but trajectories differ by
~1e-15 cm and the flux per (cell, group) is held to 1e-12 relative plus a
floor of 1e-12 of the mean entry.  With the portable functions on both sides
(the oracle's portable-math mode, pinned bit for bit to the reference linked
with them in tests/test_oracle_portable_math.py) nothing else separates them,
and the GPU meets the stricter bounds:

* the functions themselves: GPU = CPU bit for bit on 1.3 million arguments;
* tracking the oracle's particles: every census particle bit for bit, every
  tracking counter, the flux per (cell, group) within 1e-12 relative with no
  floor -- on the small decks, config1 and the benchmark deck config2;
* whole device cycles (source, population control, roulette, tracking,
  fission passes) against the reference's own portable-math run: the
  particles after every cycle init and every census bit for bit, all 13
  counters.
"""
import json
import os
import subprocess
import sys

import pytest

from helpers import DECKS
from quicksilver_gb300 import _native as N

pytestmark = pytest.mark.gpu

ROOT = DECKS.parent.parent
PM_LIB = N.LIB_PATH.parent / "libqsg_pm.so"


@pytest.fixture(scope="module")
def pm_lib():
    if not PM_LIB.exists():
        from quicksilver_gb300 import build
        build.build(portable_math=True)
    return PM_LIB


def _child(*args):
    env = dict(os.environ, QSG_LIB="pm")
    res = subprocess.run([sys.executable, str(ROOT / "tests" / "portable_math_run.py"), *map(str, args)], env=env,
                         capture_output=True, text=True, timeout=1200)
    assert res.returncode == 0, res.stdout[-2000:] + res.stderr[-4000:]
    return json.loads(res.stdout.strip().splitlines()[-1])


def test_portable_functions_gpu_equals_cpu(gpu, pm_lib):
    assert _child("functions")["bitwise_equal"]


@pytest.mark.parametrize("deck,cycles", [("t_homog", 3), ("t_scatter_octant", 3), ("t_fission", 3), ("t_nonflat", 3),
                                         ("config1", 10), ("config2", 2)])
def test_portable_math_tracking_is_bitwise(gpu, pm_lib, deck, cycles):
    out = _child("tracking", deck, cycles)
    assert out["census_bitwise"] and out["flux_worst_over_tolerance"] <= 1.0


@pytest.mark.parametrize("deck", ["t_homog", "t_escape", "t_fission", "t_nonflat", "config1", "config2"])
def test_portable_math_device_cycles_are_the_reference(gpu, pm_lib, deck):
    assert _child("cycles", deck)["particles_bitwise"]
