"""The drop-in adapter a maintainer adds to the reference -- the table
export after initMC (oracle/dropin_harness.cc, the code the integration
guide shows) -- compiled with the unmodified reference's sources and linked
against libqsg.so: for every bundled deck the export passes
qsg_problem_check (the reference's mesh self-test included), and every
table it hands the library is, bit for bit, the table this library's own
deck reader builds (node numbering aside: the reference shares nodes
between cells, so cell corners are compared as coordinates).  What the
GPU tests prove for deck-built problems therefore holds for a problem
exported from the reference's own MonteCarlo object.  Runs where the
reference's sources and the harness built from them are present, and skips
elsewhere."""
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


def _function(text: str, name: str) -> str:
    """One C++ function (signature to closing brace at column 0), whitespace collapsed."""
    m = re.search(r"^void " + name + r"\(.*?^\}", text, re.S | re.M)
    assert m, name
    return " ".join(m.group(0).split())


def test_integration_guide_shows_the_compiled_adapter():
    guide = (ROOT / "INTEGRATION.md").read_text()
    code = (ROOT / "oracle" / "dropin_harness.cc").read_text()
    assert _function(guide, "qsgExport") == _function(code, "qsgExport")
