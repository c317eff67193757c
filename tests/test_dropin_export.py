"""The drop-in adapter a maintainer adds to the reference
(oracle/dropin_harness.cc, the code the integration guide shows), compiled
with the unmodified reference's sources and linked against libqsg.so:

* the table export after initMC: for every bundled deck it passes
  qsg_problem_check (the reference's mesh self-test included), and every
  table it hands the library is, bit for bit, the table this library's own
  deck reader builds (node numbering aside: the reference shares nodes
  between cells, so cell corners are compared as coordinates) -- so what the
  GPU tests prove for deck-built problems holds for a problem exported from
  the reference's own MonteCarlo object;
* the cycle adapter's vault and tally halves around the reference's own
  first cycleInit: the particles it gathers from the processing vaults are
  the oracle's, bit for bit; scattering them into the processed vaults and
  gathering them back is exact, no vault above its size; the counters and
  flux it hands over are what the reference's Tallies then hold.

Runs where the reference's sources and the harness built from them are
present, and skips elsewhere."""
import os
import re
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

from helpers import DECKS
from quicksilver_gb300 import Deck

ROOT = Path(__file__).resolve().parent.parent
HARNESS = ROOT / "oracle" / "_ref" / "qs_dropin_harness"
sys.path.insert(0, str(ROOT / "tests" / "golden"))
from make_golden import read_dump   # noqa: E402

pytestmark = pytest.mark.skipif(not HARNESS.exists(), reason="the reference's sources or the drop-in harness are absent")

NAMES = sorted(p.stem for p in DECKS.glob("*.inp") if p.stem != "config2")   # config2: 64k cells, slow initMC


@pytest.mark.parametrize("name", NAMES)
def test_export_equals_deck_reader(name, tmp_path):
    dump = tmp_path / "export.bin"
    res = subprocess.run([str(HARNESS), "-i", str(DECKS / f"{name}.inp")], env=dict(os.environ, QS_DUMP=str(dump)),
                         capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stderr[-2000:]
    got = read_dump(dump)
    hp = Deck.from_file(DECKS / f"{name}.inp").build()
    for key, arr in got.items():
        if key in ("nodes", "cell_points"):
            continue
        want = np.array([hp.view.time_step]) if key == "time_step" else hp.array(key)
        assert arr.dtype.itemsize == want.dtype.itemsize and arr.shape == want.shape, key
        np.testing.assert_array_equal(arr.view(f"u{arr.dtype.itemsize}"), want.view(f"u{want.dtype.itemsize}"),
                                      err_msg=key)
    corners = got["nodes"].reshape(-1, 3)[got["cell_points"].reshape(-1, 14)]
    ours = hp.array("nodes").reshape(-1, 3)[hp.array("cell_points").reshape(-1, 14)]
    np.testing.assert_array_equal(corners.view(np.uint64), ours.view(np.uint64))


@pytest.mark.parametrize("name", ["t_homog", "t_fission", "t_nonflat", "config1"])
def test_cycle_adapter_vaults_and_tallies(name, tmp_path):
    from helpers import load_problem, oracle_run, sort_particles
    dump = tmp_path / "vaults.bin"
    res = subprocess.run([str(HARNESS), "-i", str(DECKS / f"{name}.inp")],
                         env=dict(os.environ, QS_DUMP=str(dump), QS_VAULTS="1"), capture_output=True, text=True,
                         timeout=300)
    assert res.returncode == 0, res.stdout[-1000:] + res.stderr[-2000:]
    got = read_dump(dump)
    _, sim, hp = load_problem(f"{name}.inp")
    run = oracle_run(hp, sim)
    run.cycle_init()
    want = run.processing()
    assert len(got["p_x"]) == len(want) > int(got["vault_size"][0])   # several vaults filled
    rec = np.zeros(len(want), want.dtype)
    for field in want.dtype.names:
        rec[field] = got["p_" + field]
    a, b = sort_particles(rec), sort_particles(want)
    for field in want.dtype.names:
        size = a[field].dtype.itemsize
        np.testing.assert_array_equal(a[field].view(f"u{size}"), b[field].view(f"u{size}"), err_msg=field)


def _block(text: str, name: str) -> str:
    """One C++ function or struct (its first line to the closing brace at
    column 0), whitespace collapsed."""
    m = re.search(r"^(?:struct |[\w:<>*& ]+ )" + name + r"\b.*?^\};?", text, re.S | re.M)
    assert m, name
    return " ".join(m.group(0).split())


@pytest.mark.parametrize("name", ["QsgExport", "qsgExport", "qsgAttach", "QsgColumns", "qsgGather",
                                  "qsgScatterCensus", "qsgAddTallies", "qsgCycleTracking"])
def test_integration_guide_shows_the_compiled_adapter(name):
    guide = (ROOT / "INTEGRATION.md").read_text()
    code = (ROOT / "oracle" / "dropin_harness.cc").read_text()
    assert _block(guide, name) == _block(code, name)
